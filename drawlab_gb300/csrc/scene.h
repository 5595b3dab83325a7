// Scene construction (scene.cpp) and the launchers of trace.cu / render.cu.
#pragma once

#include "internal.h"

namespace dl {

DevCamera make_camera(const dl_camera_desc& c);
void validate_camera(const dl_camera_desc& c);  // throws DL_ERR_INVALID_ARG
void validate_scene(const dl_mesh_desc* meshes, int32_t nm, const dl_material_desc* mats, int32_t nmat,
                    const dl_light_desc* lights, int32_t nl, const dl_camera_desc* cam);
void build_scene(dl_scene* S, const dl_mesh_desc* meshes, int32_t nm, const dl_material_desc* mats, int32_t nmat,
                 const dl_light_desc* lights, int32_t nl, const dl_camera_desc* cam);

void trace_closest_launch(dl_scene* S, const float* d_rays, int64_t n, float* d_hits, void* scratch, bool count);
void trace_any_launch(dl_scene* S, const float* d_rays, int64_t n, uint8_t* d_occ, void* scratch, bool count);
// The same queries through the renderer's own k_traverse kernels (render.cu);
// every ray starts at t = kRayEps.  Synchronises; `work` holds
// wavefront_rays_bytes(n).
size_t wavefront_rays_bytes(int64_t n);
void trace_wavefront_launch(dl_scene* S, bool any, const float* d_rays, int64_t n, float* d_hits, uint8_t* d_occ,
                            void* work);

// Device BSDF and envmap queries (query.cu); host buffers in and out.
void bsdf_query(dl_context* ctx, const dl_material_desc& m, int64_t n, const float* wi, const float* wo,
                const float* smp, float* eval, float* pdf, float* s_wo, float* s_w, float* s_eta, int32_t* s_measure);
void env_query(dl_scene* S, int64_t n, const float* xi, const float* nrm, const float* dirs, float* s_dir,
               float* s_pdf, float* s_val, float* pdf, float* val);
// Scene::sampleEmitterDirection without visibility at given points (render.cu).
void emitter_query(dl_scene* S, uint32_t flags, int64_t n, const float* pts, const float* nrm, const float* smp,
                   float* d, float* dist, float* pdf, float* spec, int32_t* light);
// L2 -> SM read bandwidth (GB/s) of L2-only loads over an L2-resident buffer.
double measure_l2_read(dl_context* ctx, int64_t bytes, int passes);

int64_t film_floats(int w, int h, int filter);
void render_run(dl_scene* S, const dl_render_opts& o, float* d_film, int64_t li_n, const int* d_xys, float* d_L,
                float* d_pos, bool count_traversal, RenderCounters* out_counters);
void resolve_film(dl_scene* S, const float* d_film, int filter, float* d_rgb);
// One-time kernel attributes of the current device (called by context creation).
void render_setup_device();

// One request of a batch: scene, options, device film (film_floats sized).
struct BatchItem {
    dl_scene* scene;
    dl_render_opts opts;
    float* d_film;
    DevCamera cam;   // the scene's camera or the request's override
};
void resolve_film_cam(const DevCamera& cam, cudaStream_t st, const float* d_film, int filter, float* d_rgb);
void render_batch(dl_context* ctx, const BatchItem* items, int n, bool count_traversal);

// Learned guiding (guide.cu).
constexpr int kGuideParams = 16560;
constexpr int kGuideImageBytes = 47808;   // fp16 weights in the tensor cores' layout, fp32 biases, W2^T, W3^T
constexpr int kGuideErrOffset = 64;       // byte offset of the error word in dl_guide::scratch
void guide_init_params(uint64_t seed, std::vector<float>& w);
void guide_upload_params(dl_guide* G, const float* host);
void guide_reserve(dl_guide* G, int64_t n);   // training buffers for batches of up to n records
void guide_gradient(dl_guide* G, const void* d_recs, int64_t n, int stride, cudaStream_t st);
void guide_adam(dl_guide* G, cudaStream_t st);
float guide_train(dl_guide* G, const void* d_recs, int64_t n, int steps);
void guide_forward(dl_guide* G, const float* d_in, float* d_out, int64_t n);
// Guided progressive render into d_film (render.cu).
void render_guided(dl_scene* S, const dl_render_opts& o, dl_guide* G, float* d_film, bool train);

// Images (image.cpp); all throw dl::Error.  Readers return RGB floats, row 0
// = the image's top row; PNG values are bytes / 255 (is_float false), PFM
// values as stored (is_float true).
void write_image(const char* path, int width, int height, const float* rgb, int format);
std::vector<float> load_pfm(const std::string& path, int& w, int& h);
std::vector<float> read_image(const std::string& path, int& w, int& h, bool& is_float);

// XML scene loading (xml.cpp): fills arrays and default render options.
struct XmlScene;
int load_xml_scene(dl_context* ctx, const char* path, dl_scene** out);

}  // namespace dl
