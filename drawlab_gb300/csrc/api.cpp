// The C ABI of include/drawlab.h: argument checks, error capture, buffer
// staging and dispatch to the scene builder, the trace kernels and the
// wavefront renderer.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>

#include "internal.h"
#include "scene.h"

namespace {

thread_local std::string g_create_error;

template <typename F>
int guard(dl_context* ctx, F&& fn) {
    try {
        if (ctx) {
            ctx->error.clear();
            cudaError_t e = cudaSetDevice(ctx->device);
            if (e != cudaSuccess) throw dl::Error(DL_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
        }
        fn();
        return DL_OK;
    } catch (const dl::Error& e) {
        if (ctx) ctx->error = e.what(); else g_create_error = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        if (ctx) ctx->error = "host allocation failed"; else g_create_error = "host allocation failed";
        return DL_ERR_OOM;
    } catch (const std::exception& e) {
        if (ctx) ctx->error = e.what(); else g_create_error = e.what();
        return DL_ERR_INVALID_ARG;
    }
}

void need(bool ok, const char* what) {
    if (!ok) throw dl::Error(DL_ERR_INVALID_ARG, what);
}
void need(bool ok, const std::string& what) {
    if (!ok) throw dl::Error(DL_ERR_INVALID_ARG, what);
}

void check_opts(const dl_render_opts* o) {
    need(o != nullptr, "opts is NULL");
    need(o->spp >= 1, "spp must be >= 1");
    need(o->rr_depth >= 0, "rr_depth must be >= 0");
    need(o->filter == DL_FILTER_GAUSSIAN || o->filter == DL_FILTER_BOX, "unknown filter");
    need(o->spp_offset >= 0, "spp_offset must be >= 0");
    need(o->max_paths_in_flight >= 0 && o->max_paths_in_flight <= ((int64_t)1 << 28), "max_paths_in_flight out of range");
    need((o->flags & ~(uint32_t)(DL_RENDER_FIX_POINT_LIGHT | DL_RENDER_POWER_LIGHT_PICK | DL_RENDER_NORMALS)) == 0,
         "unsupported render flags");
}

}  // namespace

extern "C" {

int dl_abi_version(void) { return DL_ABI_VERSION; }

const char* dl_last_error(const dl_context* ctx) { return ctx ? ctx->error.c_str() : g_create_error.c_str(); }

int dl_image_write(const char* path, int32_t width, int32_t height, const float* rgb, int32_t format) {
    g_create_error.clear();
    return guard(nullptr, [&] { dl::write_image(path, width, height, rgb, format); });
}

int dl_image_read(const char* path, int32_t* width, int32_t* height, float* rgb, int64_t capacity) {
    g_create_error.clear();
    return guard(nullptr, [&] {
        need(path != nullptr && width != nullptr && height != nullptr, "path/width/height is NULL");
        int w = 0, h = 0;
        bool is_float = false;
        std::vector<float> img = dl::read_image(path, w, h, is_float);
        *width = w;
        *height = h;
        if (rgb) {
            need(capacity >= (int64_t)img.size(), "rgb buffer too small");
            std::memcpy(rgb, img.data(), img.size() * sizeof(float));
        }
    });
}

int dl_context_create(int device, dl_context** out) {
    g_create_error.clear();
    if (!out) {
        g_create_error = "out is NULL";
        return DL_ERR_INVALID_ARG;
    }
    *out = nullptr;
    dl_context* ctx = nullptr;
    int rc = guard(nullptr, [&] {
        int n = 0;
        cudaError_t e = cudaGetDeviceCount(&n);
        if (e != cudaSuccess || n == 0) throw dl::Error(DL_ERR_CUDA, "no CUDA device available");
        if (device < 0 || device >= n) throw dl::Error(DL_ERR_INVALID_ARG, "device index out of range");
        DL_CUDA(cudaSetDevice(device));
        ctx = new dl_context();
        ctx->device = device;
        DL_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        DL_CUDA(cudaEventCreate(&ctx->ev0));
        DL_CUDA(cudaEventCreate(&ctx->ev1));
        DL_CUDA(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
        for (int i = 0; i < dl_context::kAux; i++) {
            DL_CUDA(cudaStreamCreateWithFlags(&ctx->aux[i], cudaStreamNonBlocking));
            DL_CUDA(cudaEventCreateWithFlags(&ctx->join_ev[i], cudaEventDisableTiming));
        }
        DL_CUDA(cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming));
        dl::render_setup_device();
    });
    if (rc != DL_OK) {
        delete ctx;
        return rc;
    }
    *out = ctx;
    return DL_OK;
}

int dl_context_destroy(dl_context* ctx) {
    if (!ctx) return DL_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return DL_OK;
}

int dl_scene_create_from_arrays(dl_context* ctx, const dl_mesh_desc* meshes, int32_t num_meshes,
                                const dl_material_desc* materials, int32_t num_materials,
                                const dl_light_desc* lights, int32_t num_lights, const dl_camera_desc* camera,
                                dl_scene** out) {
    if (!ctx) return DL_ERR_INVALID_ARG;
    dl_scene* S = nullptr;
    int rc = guard(ctx, [&] {
        need(out != nullptr, "out is NULL");
        *out = nullptr;
        S = new dl_scene();
        S->ctx = ctx;
        dl::build_scene(S, meshes, num_meshes, materials, num_materials, lights, num_lights, camera);
    });
    if (rc != DL_OK) {
        delete S;
        return rc;
    }
    *out = S;
    return DL_OK;
}

int dl_scene_create_from_xml(dl_context* ctx, const char* path, dl_scene** out) {
    if (!ctx) return DL_ERR_INVALID_ARG;
    int rc = DL_OK;
    int g = guard(ctx, [&] {
        need(path != nullptr && out != nullptr, "path/out is NULL");
        rc = dl::load_xml_scene(ctx, path, out);
    });
    return g != DL_OK ? g : rc;
}

int dl_scene_destroy(dl_scene* scene) {
    if (!scene) return DL_ERR_INVALID_ARG;
    cudaSetDevice(scene->ctx->device);
    cudaStreamSynchronize(scene->ctx->stream);
    delete scene;
    return DL_OK;
}

int dl_scene_get_info(const dl_scene* scene, dl_scene_info* info) {
    if (!scene || !info) return DL_ERR_INVALID_ARG;
    *info = scene->info;
    return DL_OK;
}

int dl_scene_default_opts(const dl_scene* scene, dl_render_opts* opts) {
    if (!scene || !opts) return DL_ERR_INVALID_ARG;
    *opts = scene->defaults;
    return DL_OK;
}

int dl_trace_closest_device(dl_scene* S, const float* d_rays, int64_t n, float* d_hits) {
    if (!S) return DL_ERR_INVALID_ARG;
    dl_context* ctx = S->ctx;
    return guard(ctx, [&] {
        need(n >= 0 && (n == 0 || (d_rays && d_hits)), "bad ray buffers");
        ctx->trace.occ.ensure(64);
        dl::trace_closest_launch(S, d_rays, n, d_hits, ctx->trace.occ.ptr, false);
    });
}

int dl_trace_any_device(dl_scene* S, const float* d_rays, int64_t n, uint8_t* d_occ) {
    if (!S) return DL_ERR_INVALID_ARG;
    dl_context* ctx = S->ctx;
    return guard(ctx, [&] {
        need(n >= 0 && (n == 0 || (d_rays && d_occ)), "bad ray buffers");
        ctx->trace.occ.ensure(64);
        dl::trace_any_launch(S, d_rays, n, d_occ, ctx->trace.occ.ptr, false);
    });
}

int dl_trace_closest(dl_scene* S, const float* rays, int64_t n, int32_t* prim_id, float* t, float* u, float* v) {
    if (!S) return DL_ERR_INVALID_ARG;
    dl_context* ctx = S->ctx;
    return guard(ctx, [&] {
        need(n >= 0 && (n == 0 || (rays && prim_id && t && u && v)), "bad ray buffers");
        if (n == 0) return;
        cudaStream_t st = ctx->stream;
        dl::TraceBuffers& B = ctx->trace;
        B.rays.ensure((size_t)n * 32);
        B.hits.ensure((size_t)n * 16);
        B.occ.ensure(64);
        B.stage.ensure((size_t)n * 16);
        DL_CUDA(cudaEventRecord(ctx->ev0, st));
        DL_CUDA(cudaMemcpyAsync(B.rays.ptr, rays, (size_t)n * 32, cudaMemcpyHostToDevice, st));
        dl::trace_closest_launch(S, B.rays.as<float>(), n, B.hits.as<float>(), B.occ.ptr, false);
        DL_CUDA(cudaMemcpyAsync(B.stage.ptr, B.hits.ptr, (size_t)n * 16, cudaMemcpyDeviceToHost, st));
        unsigned int err = 0;
        DL_CUDA(cudaMemcpyAsync(&err, B.occ.ptr, 4, cudaMemcpyDeviceToHost, st));
        DL_CUDA(cudaEventRecord(ctx->ev1, st));
        DL_CUDA(cudaStreamSynchronize(st));
        if (err & 4u)
            throw dl::Error(DL_ERR_QUEUE_OVERFLOW, "bounds check failed: a node or triangle index outside its array "
                                                   "(bounds-checked build)");
        if (err) throw dl::Error(DL_ERR_QUEUE_OVERFLOW, "traversal stack overflow");
        const float* h = B.stage.as<float>();
        for (int64_t i = 0; i < n; i++) {
            t[i] = h[4 * i];
            u[i] = h[4 * i + 1];
            v[i] = h[4 * i + 2];
            std::memcpy(&prim_id[i], &h[4 * i + 3], 4);
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        ctx->stats.trace_ms = ms;
    });
}

int dl_trace_any(dl_scene* S, const float* rays, int64_t n, uint8_t* occluded) {
    if (!S) return DL_ERR_INVALID_ARG;
    dl_context* ctx = S->ctx;
    return guard(ctx, [&] {
        need(n >= 0 && (n == 0 || (rays && occluded)), "bad ray buffers");
        if (n == 0) return;
        cudaStream_t st = ctx->stream;
        dl::TraceBuffers& B = ctx->trace;
        B.rays.ensure((size_t)n * 32);
        B.hits.ensure((size_t)n);
        B.occ.ensure(64);
        DL_CUDA(cudaEventRecord(ctx->ev0, st));
        DL_CUDA(cudaMemcpyAsync(B.rays.ptr, rays, (size_t)n * 32, cudaMemcpyHostToDevice, st));
        dl::trace_any_launch(S, B.rays.as<float>(), n, B.hits.as<uint8_t>(), B.occ.ptr, false);
        DL_CUDA(cudaMemcpyAsync(occluded, B.hits.ptr, (size_t)n, cudaMemcpyDeviceToHost, st));
        unsigned int err = 0;
        DL_CUDA(cudaMemcpyAsync(&err, B.occ.ptr, 4, cudaMemcpyDeviceToHost, st));
        DL_CUDA(cudaEventRecord(ctx->ev1, st));
        DL_CUDA(cudaStreamSynchronize(st));
        if (err & 4u)
            throw dl::Error(DL_ERR_QUEUE_OVERFLOW, "bounds check failed: a node or triangle index outside its array "
                                                   "(bounds-checked build)");
        if (err) throw dl::Error(DL_ERR_QUEUE_OVERFLOW, "traversal stack overflow");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        ctx->stats.trace_ms = ms;
    });
}

namespace {
// Rays through the renderer's own traversal kernels (render.cu): every ray
// must start at the renderer's constant t = kRayEps.
void trace_wavefront_host(dl_scene* S, bool any, const float* rays, int64_t n, float* hits_or_null,
                          uint8_t* occ_or_null) {
    dl_context* ctx = S->ctx;
    need(n >= 0 && n < ((int64_t)1 << 31), "bad ray count");
    for (int64_t i = 0; i < n; i++)
        need(rays[8 * i + 3] == dl::kRayEps, "wavefront traversal: every ray's tmin must be 1e-4");
    if (n == 0) return;
    cudaStream_t st = ctx->stream;
    dl::TraceBuffers& B = ctx->trace;
    B.rays.ensure((size_t)n * 32);
    B.hits.ensure((size_t)n * 16);
    B.wavefront.ensure(dl::wavefront_rays_bytes(n));
    DL_CUDA(cudaEventRecord(ctx->ev0, st));
    DL_CUDA(cudaMemcpyAsync(B.rays.ptr, rays, (size_t)n * 32, cudaMemcpyHostToDevice, st));
    dl::trace_wavefront_launch(S, any, B.rays.as<float>(), n, B.hits.as<float>(), B.hits.as<uint8_t>(),
                               B.wavefront.ptr);
    if (any) {
        DL_CUDA(cudaMemcpyAsync(occ_or_null, B.hits.ptr, (size_t)n, cudaMemcpyDeviceToHost, st));
    } else {
        DL_CUDA(cudaMemcpyAsync(hits_or_null, B.hits.ptr, (size_t)n * 16, cudaMemcpyDeviceToHost, st));
    }
    DL_CUDA(cudaEventRecord(ctx->ev1, st));
    DL_CUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->stats.trace_ms = ms;
}
}  // namespace

int dl_trace_closest_wavefront(dl_scene* S, const float* rays, int64_t n, int32_t* prim_id, float* t, float* u,
                               float* v) {
    if (!S) return DL_ERR_INVALID_ARG;
    dl_context* ctx = S->ctx;
    return guard(ctx, [&] {
        need(n >= 0 && (n == 0 || (rays && prim_id && t && u && v)), "bad ray buffers");
        std::vector<float> h((size_t)std::max<int64_t>(n, 0) * 4);
        trace_wavefront_host(S, false, rays, n, h.data(), nullptr);
        for (int64_t i = 0; i < n; i++) {
            t[i] = h[4 * i];
            u[i] = h[4 * i + 1];
            v[i] = h[4 * i + 2];
            std::memcpy(&prim_id[i], &h[4 * i + 3], 4);
        }
    });
}

int dl_trace_any_wavefront(dl_scene* S, const float* rays, int64_t n, uint8_t* occluded) {
    if (!S) return DL_ERR_INVALID_ARG;
    dl_context* ctx = S->ctx;
    return guard(ctx, [&] {
        need(n >= 0 && (n == 0 || (rays && occluded)), "bad ray buffers");
        trace_wavefront_host(S, true, rays, n, nullptr, occluded);
    });
}

int dl_bsdf_query(dl_context* ctx, const dl_material_desc* m, int64_t n, const float* wi, const float* wo,
                  const float* smp, float* eval, float* pdf, float* s_wo, float* s_weight, float* s_eta,
                  int32_t* s_measure) {
    if (!ctx) return DL_ERR_INVALID_ARG;
    return guard(ctx, [&] {
        need(m != nullptr, "material is NULL");
        need(m->type >= DL_MAT_DIFFUSE && m->type <= DL_MAT_ANISO_GGX, "unknown material type");
        need(n >= 0 && (n == 0 || (wi && wo && smp && eval && pdf && s_wo && s_weight && s_eta && s_measure)),
             "bad query buffers");
        dl::bsdf_query(ctx, *m, n, wi, wo, smp, eval, pdf, s_wo, s_weight, s_eta, s_measure);
    });
}

int dl_scene_env_query(dl_scene* S, int64_t n, const float* xi, const float* nrm, const float* dirs, float* s_dir,
                       float* s_pdf, float* s_value, float* pdf, float* value) {
    if (!S) return DL_ERR_INVALID_ARG;
    return guard(S->ctx, [&] {
        need(n >= 0 && (n == 0 || (xi && nrm && dirs && s_dir && s_pdf && s_value && pdf && value)),
             "bad query buffers");
        dl::env_query(S, n, xi, nrm, dirs, s_dir, s_pdf, s_value, pdf, value);
    });
}

int dl_scene_emitter_sample(dl_scene* S, uint32_t flags, int64_t n, const float* pts, const float* nrm,
                            const float* smp, float* d, float* dist, float* pdf, float* spec, int32_t* light) {
    if (!S) return DL_ERR_INVALID_ARG;
    return guard(S->ctx, [&] {
        need(n >= 0 && n < ((int64_t)1 << 31) && (n == 0 || (pts && nrm && smp && d && dist && pdf && spec && light)),
             "bad query buffers");
        need((flags & ~(uint32_t)(DL_RENDER_FIX_POINT_LIGHT | DL_RENDER_POWER_LIGHT_PICK)) == 0, "unsupported flags");
        dl::emitter_query(S, flags, n, pts, nrm, smp, d, dist, pdf, spec, light);
    });
}

int dl_measure_l2_read_bandwidth(dl_context* ctx, int64_t bytes, int32_t passes, double* gbs) {
    if (!ctx) return DL_ERR_INVALID_ARG;
    return guard(ctx, [&] {
        need(gbs != nullptr && bytes >= (1 << 20) && bytes <= ((int64_t)1 << 32) && passes >= 1 && passes <= 1000,
             "bad L2 probe arguments");
        DL_CUDA(cudaSetDevice(ctx->device));
        *gbs = dl::measure_l2_read(ctx, bytes, passes);
    });
}

int dl_render_film_device(dl_scene* S, const dl_render_opts* opts, float* d_film) {
    if (!S) return DL_ERR_INVALID_ARG;
    return guard(S->ctx, [&] {
        check_opts(opts);
        need(d_film != nullptr, "d_film is NULL");
        dl::render_run(S, *opts, d_film, 0, nullptr, nullptr, nullptr, false, nullptr);
    });
}

int dl_render_film(dl_scene* S, const dl_render_opts* opts, float* film_out) {
    if (!S) return DL_ERR_INVALID_ARG;
    dl_context* ctx = S->ctx;
    return guard(ctx, [&] {
        check_opts(opts);
        need(film_out != nullptr, "film_out is NULL");
        int64_t nf = dl::film_floats(S->dev.cam.w, S->dev.cam.h, opts->filter);
        ctx->render.film.ensure((size_t)nf * 4);
        dl::render_run(S, *opts, ctx->render.film.as<float>(), 0, nullptr, nullptr, nullptr, false, nullptr);
        DL_CUDA(cudaMemcpyAsync(film_out, ctx->render.film.ptr, (size_t)nf * 4, cudaMemcpyDeviceToHost, ctx->stream));
        DL_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int dl_render(dl_scene* S, const dl_render_opts* opts, float* rgb_out) {
    if (!S) return DL_ERR_INVALID_ARG;
    dl_context* ctx = S->ctx;
    return guard(ctx, [&] {
        check_opts(opts);
        need(rgb_out != nullptr, "rgb_out is NULL");
        int64_t nf = dl::film_floats(S->dev.cam.w, S->dev.cam.h, opts->filter);
        size_t nrgb = (size_t)S->dev.cam.w * S->dev.cam.h * 3;
        ctx->render.film.ensure((size_t)nf * 4);
        ctx->render.rgb.ensure(nrgb * 4);
        dl::render_run(S, *opts, ctx->render.film.as<float>(), 0, nullptr, nullptr, nullptr, false, nullptr);
        dl::resolve_film(S, ctx->render.film.as<float>(), opts->filter, ctx->render.rgb.as<float>());
        DL_CUDA(cudaMemcpyAsync(rgb_out, ctx->render.rgb.ptr, nrgb * 4, cudaMemcpyDeviceToHost, ctx->stream));
        DL_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int dl_li(dl_scene* S, const dl_render_opts* opts, int64_t n, const int32_t* xys, float* L_out, float* pos_out) {
    if (!S) return DL_ERR_INVALID_ARG;
    dl_context* ctx = S->ctx;
    return guard(ctx, [&] {
        need(opts != nullptr, "opts is NULL");
        need(n >= 0 && (n == 0 || (xys && L_out)), "bad path buffers");
        need(n < ((int64_t)1 << 31), "at most 2^31 - 1 paths per call");
        if (n == 0) return;
        const dl::DevCamera& cam = S->dev.cam;
        for (int64_t i = 0; i < n; i++)
            need(xys[3 * i] >= 0 && xys[3 * i] < cam.w && xys[3 * i + 1] >= 0 && xys[3 * i + 1] < cam.h &&
                     xys[3 * i + 2] >= 0,
                 "path (x, y, s) out of range");
        dl_render_opts o = *opts;
        o.spp = 1;
        check_opts(&o);
        cudaStream_t st = ctx->stream;
        dl::RenderBuffers& B = ctx->render;
        B.li_xys.ensure((size_t)n * 12);
        B.li_out.ensure((size_t)n * 12);
        B.li_pos.ensure((size_t)n * 8);
        DL_CUDA(cudaMemcpyAsync(B.li_xys.ptr, xys, (size_t)n * 12, cudaMemcpyHostToDevice, st));
        dl::render_run(S, o, nullptr, n, B.li_xys.as<int>(), B.li_out.as<float>(), B.li_pos.as<float>(), false,
                       nullptr);
        DL_CUDA(cudaMemcpyAsync(L_out, B.li_out.ptr, (size_t)n * 12, cudaMemcpyDeviceToHost, st));
        if (pos_out) DL_CUDA(cudaMemcpyAsync(pos_out, B.li_pos.ptr, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
        DL_CUDA(cudaStreamSynchronize(st));
    });
}

int dl_render_traversal_counts(dl_scene* S, const dl_render_opts* opts, dl_traversal_counts* out) {
    if (!S) return DL_ERR_INVALID_ARG;
    dl_context* ctx = S->ctx;
    return guard(ctx, [&] {
        check_opts(opts);
        need(out != nullptr, "out is NULL");
        int64_t nf = dl::film_floats(S->dev.cam.w, S->dev.cam.h, opts->filter);
        ctx->render.film.ensure((size_t)nf * 4);
        dl::RenderCounters rc;
        dl::render_run(S, *opts, ctx->render.film.as<float>(), 0, nullptr, nullptr, nullptr, true, &rc);
        out->extension_rays = (int64_t)rc.stat_ext;
        out->shadow_rays = (int64_t)rc.stat_shadow;
        out->extension_node_visits = (int64_t)rc.stat_nodes_ext;
        out->extension_triangle_tests = (int64_t)rc.stat_tris_ext;
        out->shadow_node_visits = (int64_t)rc.stat_nodes_sh;
        out->shadow_triangle_tests = (int64_t)rc.stat_tris_sh;
    });
}

}  // extern "C"

namespace {

// Validated batch items; requests without a device film get one in the
// context's batch film buffer (offsets in floats in `film_off`, -1 when the
// caller gave one).  trial_spp >= 0 overrides every request's spp (0: an
// eighth of it, at least 1).
std::vector<dl::BatchItem> batch_items(dl_context* ctx, const dl_request* reqs, int32_t n, bool outputs,
                                       int trial_spp, std::vector<int64_t>& film_off) {
    need(n >= 0 && (n == 0 || reqs != nullptr), "bad request array");
    need(n <= (1 << 20), "at most 2^20 requests per batch");
    std::vector<dl::BatchItem> items((size_t)n);
    film_off.assign((size_t)n, -1);
    int64_t floats = 0;
    for (int32_t r = 0; r < n; r++) {
        const dl_request& q = reqs[r];
        need(q.scene != nullptr, "request " + std::to_string(r) + ": scene is NULL");
        need(q.scene->ctx == ctx, "request " + std::to_string(r) + ": scene belongs to another context");
        check_opts(&q.opts);
        if (outputs) need(q.rgb || q.film_device, "request " + std::to_string(r) + ": no output");
        items[r].scene = q.scene;
        items[r].opts = q.opts;
        items[r].cam = q.scene->dev.cam;
        if (q.camera) {
            const dl_camera_desc& c = *q.camera;
            try {
                dl::validate_camera(c);
            } catch (const dl::Error& e) {
                throw dl::Error(DL_ERR_INVALID_ARG, "request " + std::to_string(r) + ": " + e.what());
            }
            items[r].cam = dl::make_camera(c);
        }
        if (trial_spp >= 0) items[r].opts.spp = trial_spp > 0 ? trial_spp : std::max(1, q.opts.spp / 8);
        items[r].d_film = outputs ? q.film_device : nullptr;
        if (!items[r].d_film) {
            film_off[r] = floats;
            floats += dl::film_floats(items[r].cam.w, items[r].cam.h, q.opts.filter);
        }
    }
    ctx->render.batch_films.ensure((size_t)std::max<int64_t>(floats, 1) * 4);
    for (int32_t r = 0; r < n; r++)
        if (film_off[r] >= 0) items[r].d_film = ctx->render.batch_films.as<float>() + film_off[r];
    return items;
}

}  // namespace

extern "C" {

int dl_render_batch(dl_context* ctx, const dl_request* reqs, int32_t n) {
    if (!ctx) return DL_ERR_INVALID_ARG;
    return guard(ctx, [&] {
        std::vector<int64_t> off;
        std::vector<dl::BatchItem> items = batch_items(ctx, reqs, n, true, -1, off);
        if (n == 0) return;
        dl::render_batch(ctx, items.data(), n, false);
        size_t maxrgb = 0;
        for (int32_t r = 0; r < n; r++)
            if (reqs[r].rgb) maxrgb = std::max(maxrgb, (size_t)items[r].cam.w * items[r].cam.h * 3);
        ctx->render.rgb.ensure(std::max<size_t>(maxrgb, 1) * 4);
        for (int32_t r = 0; r < n; r++) {
            if (!reqs[r].rgb) continue;
            size_t nrgb = (size_t)items[r].cam.w * items[r].cam.h * 3;
            dl::resolve_film_cam(items[r].cam, ctx->stream, items[r].d_film, items[r].opts.filter,
                                 ctx->render.rgb.as<float>());
            DL_CUDA(cudaMemcpyAsync(reqs[r].rgb, ctx->render.rgb.ptr, nrgb * 4, cudaMemcpyDeviceToHost, ctx->stream));
            DL_CUDA(cudaStreamSynchronize(ctx->stream));
        }
    });
}

int dl_context_get_tune(const dl_context* ctx, dl_tune_params* out) {
    if (!ctx || !out) return DL_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    out->paths_in_flight = ctx->tune.paths_in_flight;
    out->traverse_ctas_per_sm = ctx->tune.trav_ctas_per_sm;
    out->shade_ctas_per_sm = ctx->tune.shade_ctas_per_sm;
    out->iterations_per_graph = ctx->tune.iters_per_graph;
    out->shade_threads = ctx->tune.shade_threads;
    return DL_OK;
}

int dl_context_set_tune(dl_context* ctx, const dl_tune_params* t) {
    if (!ctx) return DL_ERR_INVALID_ARG;
    return guard(ctx, [&] {
        need(t != nullptr, "tune is NULL");
        need(t->paths_in_flight >= 32 && t->paths_in_flight <= ((int64_t)1 << 28), "paths_in_flight out of range");
        need(t->traverse_ctas_per_sm >= 1 && t->traverse_ctas_per_sm <= 16, "traverse_ctas_per_sm out of range");
        need(t->shade_ctas_per_sm >= 1 && t->shade_ctas_per_sm <= 64, "shade_ctas_per_sm out of range");
        need(t->iterations_per_graph >= 2 && t->iterations_per_graph <= 8 && t->iterations_per_graph % 2 == 0,
             "iterations_per_graph must be 2, 4, 6 or 8");
        need(t->shade_threads == 0 || t->shade_threads == 64 || t->shade_threads == 128 || t->shade_threads == 256,
             "shade_threads must be 64, 128 or 256 (0: 128)");
        ctx->tune.paths_in_flight = t->paths_in_flight;
        ctx->tune.trav_ctas_per_sm = t->traverse_ctas_per_sm;
        ctx->tune.shade_ctas_per_sm = t->shade_ctas_per_sm;
        ctx->tune.iters_per_graph = t->iterations_per_graph;
        ctx->tune.shade_threads = t->shade_threads == 0 ? 128 : t->shade_threads;
    });
}

int dl_autotune(dl_context* ctx, const dl_request* reqs, int32_t n, int32_t trial_spp, dl_tune_params* out,
                int32_t* trials) {
    if (!ctx) return DL_ERR_INVALID_ARG;
    return guard(ctx, [&] {
        need(trial_spp >= 0, "trial_spp must be >= 0");
        need(n >= 1, "autotune needs at least one request");
        std::vector<int64_t> off;
        std::vector<dl::BatchItem> items = batch_items(ctx, reqs, n, false, trial_spp, off);
        for (auto& it : items) it.opts.max_paths_in_flight = 0;  // the pool size is what is tuned
        const bool timing = ctx->kernel_timing;
        ctx->kernel_timing = false;
        int count = 0;
        auto time_of = [&](const dl::TuneParams& tp) {
            ctx->tune = tp;
            dl::render_batch(ctx, items.data(), n, false);
            count++;
            return ctx->stats.render_ms;
        };
        dl::TuneParams best = ctx->tune;
        try {
            (void)time_of(best);  // warm-up: buffers, graph
            double best_ms = time_of(best);
            auto search = [&](auto setter, std::initializer_list<int64_t> values) {
                for (int64_t v : values) {
                    dl::TuneParams tp = best;
                    setter(tp, v);
                    double ms = time_of(tp);
                    if (ms < best_ms) {
                        best_ms = ms;
                        best = tp;
                    }
                }
            };
            search([](dl::TuneParams& t, int64_t v) { t.paths_in_flight = v; },
                   {(int64_t)1 << 20, (int64_t)1 << 21, (int64_t)1 << 22, (int64_t)1 << 23, (int64_t)1 << 24,
                    (int64_t)1 << 25});
            search([](dl::TuneParams& t, int64_t v) { t.trav_ctas_per_sm = (int)v; }, {4, 6, 8});
            search([](dl::TuneParams& t, int64_t v) { t.shade_ctas_per_sm = (int)v; }, {8, 16, 32});
            // block size of the shading kernels at the same threads per SM
            search(
                [&](dl::TuneParams& t, int64_t v) {
                    t.shade_ctas_per_sm = std::max(1, std::min(64, best.shade_ctas_per_sm * best.shade_threads / (int)v));
                    t.shade_threads = (int)v;
                },
                {64, 256});
            search([](dl::TuneParams& t, int64_t v) { t.iters_per_graph = (int)v; }, {2, 4, 8});
        } catch (...) {
            ctx->tune = best;
            ctx->kernel_timing = timing;
            throw;
        }
        ctx->tune = best;
        ctx->kernel_timing = timing;
        if (trials) *trials = count;
        if (out) {
            std::memset(out, 0, sizeof(*out));
            out->paths_in_flight = best.paths_in_flight;
            out->traverse_ctas_per_sm = best.trav_ctas_per_sm;
            out->shade_ctas_per_sm = best.shade_ctas_per_sm;
            out->iterations_per_graph = best.iters_per_graph;
            out->shade_threads = best.shade_threads;
        }
    });
}

int dl_guide_default_config(dl_guide_config* cfg) {
    if (!cfg) return DL_ERR_INVALID_ARG;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->learning_rate = 2e-3f;
    cfg->guide_fraction = 0.5f;
    cfg->batch = 131072;
    cfg->steps_per_pass = 16;
    cfg->max_guided_depth = 6;
    cfg->seed = 1;
    return DL_OK;
}

namespace {
// The guide's error word: a tensor-core wait in a training or network
// kernel that ran out sets it.
void guide_err_reset(dl_guide* G, cudaStream_t st) {
    DL_CUDA(cudaMemsetAsync(G->scratch.as<char>() + dl::kGuideErrOffset, 0, 4, st));
}
void guide_err_check(dl_guide* G, cudaStream_t st) {
    unsigned err = 0;
    DL_CUDA(cudaMemcpyAsync(&err, G->scratch.as<char>() + dl::kGuideErrOffset, 4, cudaMemcpyDeviceToHost, st));
    DL_CUDA(cudaStreamSynchronize(st));
    if (err) throw dl::Error(DL_ERR_TIMEOUT, "tensor-core wait timed out in a network kernel");
}
}  // namespace

int dl_guide_create(dl_context* ctx, const dl_guide_config* cfg, dl_guide** out) {
    if (!ctx) return DL_ERR_INVALID_ARG;
    dl_guide* G = nullptr;
    int rc = guard(ctx, [&] {
        need(cfg != nullptr && out != nullptr, "cfg/out is NULL");
        need(cfg->learning_rate > 0.f && cfg->learning_rate < 1.f, "learning_rate out of range");
        need(cfg->guide_fraction >= 0.f && cfg->guide_fraction < 1.f, "guide_fraction must be in [0, 1)");
        need(cfg->batch >= 16 && cfg->batch <= (1 << 24), "batch out of range");
        need(cfg->steps_per_pass >= 0 && cfg->steps_per_pass <= 1024, "steps_per_pass out of range");
        need(cfg->max_guided_depth >= 0 && cfg->max_guided_depth <= 1 << 20, "max_guided_depth out of range");
        *out = nullptr;
        G = new dl_guide();
        G->ctx = ctx;
        G->cfg = *cfg;
        const size_t pb = dl::kGuideParams * 4;
        for (dl::DevBuf* b : {&G->w32, &G->grad, &G->m, &G->v}) b->ensure(pb);
        G->w16.ensure(dl::kGuideParams * 2);
        G->image.ensure(dl::kGuideImageBytes);
        G->scratch.ensure(256);
        // training overlaps the next render pass; at the highest priority its
        // few short kernels are scheduled ahead of the pass's blocks, so the
        // pass samples with the updated network early on
        int lo_prio = 0, hi_prio = 0;
        DL_CUDA(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio));
        DL_CUDA(cudaStreamCreateWithPriority(&G->train_stream, cudaStreamNonBlocking, hi_prio));
        for (int k = 0; k < 2; k++) {
            DL_CUDA(cudaEventCreateWithFlags(&G->pass_done[k], cudaEventDisableTiming));
            DL_CUDA(cudaEventCreateWithFlags(&G->train_done[k], cudaEventDisableTiming));
        }
        DL_CUDA(cudaEventCreate(&G->t0));
        DL_CUDA(cudaEventCreate(&G->t1));
        for (dl::DevBuf* b : {&G->grad, &G->m, &G->v}) DL_CUDA(cudaMemsetAsync(b->ptr, 0, pb, ctx->stream));
        std::vector<float> w;
        dl::guide_init_params(cfg->seed, w);
        dl::guide_upload_params(G, w.data());
        DL_CUDA(cudaStreamSynchronize(ctx->stream));
    });
    if (rc != DL_OK) {
        delete G;
        return rc;
    }
    *out = G;
    return DL_OK;
}

int dl_guide_destroy(dl_guide* G) {
    if (!G) return DL_ERR_INVALID_ARG;
    cudaSetDevice(G->ctx->device);
    cudaStreamSynchronize(G->ctx->stream);
    delete G;
    return DL_OK;
}

int dl_guide_get_params(const dl_guide* G, float* params) {
    if (!G || !params) return DL_ERR_INVALID_ARG;
    dl_context* ctx = G->ctx;
    return guard(ctx, [&] {
        DL_CUDA(cudaMemcpyAsync(params, G->w32.ptr, dl::kGuideParams * 4, cudaMemcpyDeviceToHost, ctx->stream));
        DL_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int dl_guide_set_params(dl_guide* G, const float* params) {
    if (!G) return DL_ERR_INVALID_ARG;
    return guard(G->ctx, [&] {
        need(params != nullptr, "params is NULL");
        for (int i = 0; i < dl::kGuideParams; i++) need(std::isfinite(params[i]), "params must be finite");
        dl::guide_upload_params(G, params);
        DL_CUDA(cudaStreamSynchronize(G->ctx->stream));
    });
}

int dl_guide_forward(dl_guide* G, int64_t n, const float* inputs, float* outputs) {
    if (!G) return DL_ERR_INVALID_ARG;
    dl_context* ctx = G->ctx;
    return guard(ctx, [&] {
        need(n >= 0 && n < ((int64_t)1 << 31) && (n == 0 || (inputs && outputs)), "bad buffers");
        if (n == 0) return;
        G->io_in.ensure((size_t)n * 6 * 4);
        G->io_out.ensure((size_t)n * 40 * 4);
        DL_CUDA(cudaMemcpyAsync(G->io_in.ptr, inputs, (size_t)n * 24, cudaMemcpyHostToDevice, ctx->stream));
        DL_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
        dl::guide_forward(G, G->io_in.as<float>(), G->io_out.as<float>(), n);
        DL_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
        DL_CUDA(cudaMemcpyAsync(outputs, G->io_out.ptr, (size_t)n * 160, cudaMemcpyDeviceToHost, ctx->stream));
        unsigned err = 0;
        DL_CUDA(cudaMemcpyAsync(&err, G->scratch.as<char>() + dl::kGuideErrOffset, 4, cudaMemcpyDeviceToHost,
                                ctx->stream));
        DL_CUDA(cudaStreamSynchronize(ctx->stream));
        if (err) throw dl::Error(DL_ERR_TIMEOUT, "tensor-core wait timed out in the network kernel");
        float ms = 0.f;
        DL_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        ctx->stats.guide_ms = ms;
    });
}

int dl_guide_gradient(dl_guide* G, int64_t n, const float* records, float* grad, float* loss) {
    if (!G) return DL_ERR_INVALID_ARG;
    dl_context* ctx = G->ctx;
    return guard(ctx, [&] {
        need(n >= 1 && n <= (1 << 24) && records && grad, "bad buffers");
        G->recs.ensure((size_t)n * 48);
        DL_CUDA(cudaMemcpyAsync(G->recs.ptr, records, (size_t)n * 48, cudaMemcpyHostToDevice, ctx->stream));
        DL_CUDA(cudaMemsetAsync(G->grad.ptr, 0, dl::kGuideParams * 4, ctx->stream));
        guide_err_reset(G, ctx->stream);
        dl::guide_reserve(G, n);
        DL_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
        dl::guide_gradient(G, G->recs.ptr, n, 1, ctx->stream);
        DL_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
        DL_CUDA(cudaMemcpyAsync(grad, G->grad.ptr, dl::kGuideParams * 4, cudaMemcpyDeviceToHost, ctx->stream));
        float l = 0.f;
        DL_CUDA(cudaMemcpyAsync(&l, G->scratch.as<float>() + 1, 4, cudaMemcpyDeviceToHost, ctx->stream));
        DL_CUDA(cudaMemsetAsync(G->grad.ptr, 0, dl::kGuideParams * 4, ctx->stream));
        DL_CUDA(cudaStreamSynchronize(ctx->stream));
        guide_err_check(G, ctx->stream);
        if (loss) *loss = l;
        float ms = 0.f;
        DL_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        ctx->stats.guide_ms = ms;
    });
}

int dl_guide_train(dl_guide* G, int64_t n, const float* records, int32_t steps, float* loss) {
    if (!G) return DL_ERR_INVALID_ARG;
    dl_context* ctx = G->ctx;
    return guard(ctx, [&] {
        need(n >= 1 && n <= (1 << 24) && records, "bad buffers");
        need(steps >= 0 && steps <= 100000, "steps out of range");
        G->recs.ensure((size_t)n * 48);
        DL_CUDA(cudaMemcpyAsync(G->recs.ptr, records, (size_t)n * 48, cudaMemcpyHostToDevice, ctx->stream));
        guide_err_reset(G, ctx->stream);
        float l = dl::guide_train(G, G->recs.ptr, n, steps);
        guide_err_check(G, ctx->stream);
        if (loss) *loss = l;
    });
}

int dl_render_guided(dl_scene* S, const dl_render_opts* opts, dl_guide* G, int32_t train, float* rgb_out) {
    if (!S) return DL_ERR_INVALID_ARG;
    dl_context* ctx = S->ctx;
    return guard(ctx, [&] {
        check_opts(opts);
        need(G != nullptr && G->ctx == ctx, "guide is NULL or belongs to another context");
        need(!(opts->flags & DL_RENDER_NORMALS), "the normals integrator has no guided form");
        need(rgb_out != nullptr, "rgb_out is NULL");
        int64_t nf = dl::film_floats(S->dev.cam.w, S->dev.cam.h, opts->filter);
        size_t nrgb = (size_t)S->dev.cam.w * S->dev.cam.h * 3;
        ctx->render.film.ensure((size_t)nf * 4);
        ctx->render.rgb.ensure(nrgb * 4);
        guide_err_reset(G, ctx->stream);
        dl::render_guided(S, *opts, G, ctx->render.film.as<float>(), train != 0);
        guide_err_check(G, ctx->stream);
        dl::resolve_film(S, ctx->render.film.as<float>(), opts->filter, ctx->render.rgb.as<float>());
        DL_CUDA(cudaMemcpyAsync(rgb_out, ctx->render.rgb.ptr, nrgb * 4, cudaMemcpyDeviceToHost, ctx->stream));
        DL_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int dl_context_set_kernel_timing(dl_context* ctx, int enabled) {
    if (!ctx) return DL_ERR_INVALID_ARG;
    ctx->kernel_timing = enabled != 0;
    return DL_OK;
}

int dl_stats_get(const dl_context* ctx, dl_stats* stats) {
    if (!ctx || !stats) return DL_ERR_INVALID_ARG;
    *stats = ctx->stats;
    return DL_OK;
}

}  // extern "C"
