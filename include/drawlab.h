/*
 * drawlab.h -- C ABI of the GB300 wavefront path tracer.
 *
 * Plain C types only (pointers, sizes, PODs): any FFI (ctypes, cgo, JNI,
 * N-API) can bind it.  Every entry point returns an int status (DL_OK on
 * success); dl_last_error() gives the message of the last failure on a
 * context.  No C++ exception crosses this boundary.
 *
 * The reference (xuxmin/DrawLab) exposes the same path as C++ virtual
 * interfaces.  Each entry point below names the reference interface it
 * stands in for (paths are relative to the reference project root).
 *
 * Threading: calls on one dl_context are serialised by the caller.  Distinct
 * contexts are independent.  One CUDA stream per context.
 */
#ifndef DRAWLAB_H
#define DRAWLAB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DL_ABI_VERSION 8

/* ------------------------------------------------------------------ status */
enum dl_status {
    DL_OK = 0,
    DL_ERR_INVALID_ARG = 1,
    DL_ERR_OOM = 2,
    DL_ERR_CUDA = 3,
    DL_ERR_TIMEOUT = 4,
    DL_ERR_QUEUE_OVERFLOW = 5,
    DL_ERR_PARSE = 6,
    DL_ERR_UNSUPPORTED = 7,
    DL_ERR_IO = 8
};

typedef struct dl_context dl_context;
typedef struct dl_scene dl_scene;

/* ------------------------------------------------------- scene descriptors */

/* Triangle mesh.  Stands in for drawlab::Mesh (include/tracer/mesh.h:20-252):
 * positions m_V, normals m_N, texcoords m_UV, faces m_F.  normals/texcoords
 * may be NULL.  A mesh carries one material and, optionally, one area light
 * (Mesh::addChild, src/tracer/mesh/mesh.cpp:47-69). */
typedef struct dl_mesh_desc {
    const float* positions;   /* num_vertices x 3 */
    const float* normals;     /* num_vertices x 3, or NULL */
    const float* texcoords;   /* num_vertices x 2, or NULL */
    const uint32_t* indices;  /* num_triangles x 3 */
    int64_t num_vertices;
    int64_t num_triangles;
    int32_t material;         /* index into the material array */
    int32_t light;            /* index of the area light bound to it, or -1 */
} dl_mesh_desc;

/* BSDF plugins (include/tracer/bsdf.h:46-110), XML type strings in brackets. */
enum dl_material_type {
    DL_MAT_DIFFUSE = 0,     /* "diffuse"    src/tracer/bsdf/diffuse.cpp */
    DL_MAT_MIRROR = 1,      /* "mirror"     src/tracer/bsdf/mirror.cpp */
    DL_MAT_DIELECTRIC = 2,  /* "dielectric" src/tracer/bsdf/dielectric.cpp */
    DL_MAT_MICROFACET = 3,  /* "microfacet" src/tracer/bsdf/microfacet.cpp (Beckmann) */
    DL_MAT_ANISO_GGX = 4    /* "aniso_ggx"  src/optix/cuda/material/aniso_ggx.cu */
};

/* A bitmap texture: `height` rows of `width` RGB floats; row k is sampled
 * around texture coordinate t = (k + 0.5) / height, column j around
 * s = (j + 0.5) / width -- the texel order the reference uploads (8-bit
 * images top row first, float images bottom row first,
 * src/tracer/texture/bitmap.cpp:60-98).  rgb NULL: no texture. */
typedef struct dl_texture_desc {
    const float* rgb;
    int32_t width;
    int32_t height;
} dl_texture_desc;

typedef struct dl_material_desc {
    int32_t type;         /* dl_material_type */
    float albedo[3];      /* diffuse albedo | microfacet kd | aniso_ggx pd */
    float specular[3];    /* aniso_ggx ps */
    float alpha[2];       /* microfacet alpha in [0]; aniso_ggx (ax, ay) */
    float int_ior;        /* dielectric / microfacet interior IOR */
    float ext_ior;        /* dielectric / microfacet exterior IOR */
    /* Bitmap textures (the reference reads them in its OptiX path only:
     * src/optix/cuda/material/diffuse.cu:15-20, aniso_ggx.cu:19-35,
     * src/optix/cuda/shader_common.h:38-143), looked up at the hit's
     * interpolated texture coordinates (the mesh's texcoords; (0, 0) without
     * them) with bilinear filtering and wrap addressing.  They replace the
     * constants above. */
    dl_texture_desc albedo_texture;    /* diffuse albedo | aniso_ggx pd */
    dl_texture_desc specular_texture;  /* aniso_ggx ps */
    dl_texture_desc alpha_texture;     /* aniso_ggx (ax, ay) = (R, G) */
    dl_texture_desc normal_texture;    /* aniso_ggx world-space shading normal: normalize(2 rgb - 1) */
    dl_texture_desc tangent_texture;   /* aniso_ggx world-space shading tangent: normalize(2 rgb - 1) */
} dl_material_desc;

/* Emitter plugins (include/tracer/emitter.h:7-117). */
enum dl_light_type {
    DL_LIGHT_AREA = 0,    /* "area"   src/tracer/emitter/area.cpp */
    DL_LIGHT_POINT = 1,   /* "point"  src/tracer/emitter/point.cpp */
    DL_LIGHT_ENVMAP = 2   /* "envmap" src/tracer/emitter/envmap.cpp + include/optix/light/envmap.h */
};

/* The order of the light array is the emitter order of the scene: the
 * uniform emitter pick of Scene::sampleEmitterDirection
 * (src/tracer/scene/scene.cpp:148-163) indexes it. */
typedef struct dl_light_desc {
    int32_t type;          /* dl_light_type */
    int32_t mesh;          /* area: index of the emitting mesh */
    float radiance[3];     /* area radiance | point intensity */
    float position[3];     /* point position */
    /* envmap: env_height x env_width x 3 floats, latitude-longitude.  Row 0
     * is the +y pole (theta = 0), the last row the -y pole; column u covers
     * phi = atan2(z, x) = 2 pi u - pi (include/optix/light/envmap.h:26-30).
     * At most one envmap per scene (src/tracer/scene/scene.cpp:72-78). */
    const float* env_rgb;
    int32_t env_width;
    int32_t env_height;
    float env_scale;       /* envmap "scale" (default 1) */
    int32_t env_visual;    /* envmap "visual": seen by camera rays (default 1) */
    float env_background[3]; /* what camera rays that miss see when visual = 0:
                                the scene's "bg_color" (scene.cpp:7, miss.cu:20-27) */
} dl_light_desc;

enum dl_camera_type {
    DL_CAMERA_VIRTUAL = 0,     /* "virtual" src/tracer/camera/virtual.cpp:14-123 */
    DL_CAMERA_PERSPECTIVE = 1, /* "perspective" src/tracer/camera/perspective.cpp:19-100:
                                  pinhole through a camera-to-world transform */
    DL_CAMERA_OPENCV = 2       /* "opencv" src/tracer/camera/opencv.cpp:8-87 (host) and
                                  include/optix/camera/opencv.h:24-47 (rays): intrinsics
                                  fx, fy, cx, cy and a world-to-camera extrinsic */
};

typedef struct dl_camera_desc {
    int32_t type;          /* dl_camera_type */
    int32_t width;
    int32_t height;
    float eye[3];          /* virtual */
    float lookat[3];       /* virtual */
    float up[3];           /* virtual */
    float fov;             /* virtual: vertical field of view; perspective: horizontal
                              field of view (degrees) */
    float transform[16];   /* row-major 4x4.  perspective: camera-to-world ("toWorld",
                              identity when absent); opencv: the world-to-camera
                              "extrinsic" */
    float near_clip;       /* perspective: near and far clip distances (reference */
    float far_clip;        /*   defaults 1e-4 and 1e4); camera rays span [near, far] / d.z */
    float fx, fy, cx, cy;  /* opencv intrinsics (pixels) */
} dl_camera_desc;

/* ------------------------------------------------------------------ context */

/* Create a context on CUDA device `device` (one stream, device memory owned
 * by the context).  No reference counterpart: the reference owns one OptiX
 * DeviceContext per renderer (src/optix/host/device_context.cpp:55). */
int dl_context_create(int device, dl_context** out);
int dl_context_destroy(dl_context* ctx);
/* Message of the last failed call on ctx ("" if none).  Valid until the next
 * call on ctx.  ctx may be NULL for failures of dl_context_create. */
const char* dl_last_error(const dl_context* ctx);
/* ABI version compiled into the library (DL_ABI_VERSION). */
int dl_abi_version(void);

/* -------------------------------------------------------------------- scene */

/* Build a scene from arrays: uploads geometry, builds the SAH BVH on the
 * host and copies it to the device.  Replaces loadFromXML + Scene::addChild +
 * Scene::activate + OCTree::build (src/core/parser/parser.cpp:19-387,
 * src/tracer/scene/scene.cpp:19-106, src/tracer/accel/octree.cpp:135-151). */
int dl_scene_create_from_arrays(dl_context* ctx,
                                const dl_mesh_desc* meshes, int32_t num_meshes,
                                const dl_material_desc* materials, int32_t num_materials,
                                const dl_light_desc* lights, int32_t num_lights,
                                const dl_camera_desc* camera,
                                dl_scene** out);

/* Load a scene in the reference's XML format (mitsuba-style tags: scene,
 * mesh, bsdf, emitter, camera, integrator, sampler, rfilter; properties and
 * transforms).  Replaces loadFromXML (src/core/parser/parser.cpp:19-387).
 * The sampler's sampleCount and the rfilter become the scene's default
 * render options (see dl_scene_default_opts). */
int dl_scene_create_from_xml(dl_context* ctx, const char* path, dl_scene** out);
int dl_scene_destroy(dl_scene* scene);

typedef struct dl_scene_info {
    int64_t num_triangles;
    int64_t num_bvh_nodes;
    int32_t num_meshes;
    int32_t num_materials;
    int32_t num_lights;
    int32_t width;
    int32_t height;
    int32_t bvh_depth;
    double bvh_build_seconds;
    double bvh_sah_cost;
    int64_t device_bytes;
} dl_scene_info;
int dl_scene_get_info(const dl_scene* scene, dl_scene_info* info);

/* ---------------------------------------------------------------- tracing */

/* Rays are packed 8 floats each: ox, oy, oz, tmin, dx, dy, dz, tmax.
 * Reference: Ray3f (include/core/math/ray.h:22-81); M_EPSILON = 1e-4 is the
 * reference's default tmin. */

/* Closest hit.  Replaces Accel::rayIntersect(ray, its, false) / OCTree
 * (include/tracer/accel.h:52, src/tracer/accel/octree.cpp:53-110,153-212)
 * with the Moller-Trumbore test of Mesh::rayIntersect
 * (src/tracer/mesh/mesh.cpp:180-220).  prim_id is the global triangle index
 * (meshes concatenated in order), -1 on a miss; t, u, v as the reference
 * computes them.  Host buffers. */
int dl_trace_closest(dl_scene* scene, const float* rays, int64_t n,
                     int32_t* prim_id, float* t, float* u, float* v);

/* Any hit (shadow query).  Replaces Accel::rayIntersect(ray, its, true) /
 * OCTree::recursiveAnyhit (src/tracer/accel/octree.cpp:112-133). */
int dl_trace_any(dl_scene* scene, const float* rays, int64_t n, uint8_t* occluded);

/* Device-pointer forms of the two calls above (inputs already resident in
 * device memory; launched on the context stream, which the call leaves
 * unsynchronised).  hits: n x {t, u, v, prim_id bits} float4. */
int dl_trace_closest_device(dl_scene* scene, const float* d_rays, int64_t n, float* d_hits);
int dl_trace_any_device(dl_scene* scene, const float* d_rays, int64_t n, uint8_t* d_occluded);

/* The same two queries (same reference functions, same outputs) traced by
 * the renderer's own persistent wavefront traversal kernels -- the kernels
 * dl_render launches for extension and shadow rays -- instead of the
 * stand-alone ray-batch kernels above.  Those kernels start every ray at
 * the renderer's constant t = 1e-4 (the reference's Epsilon, scene.cpp:
 * 165-169), so every ray's tmin must be 1e-4, else DL_ERR_INVALID_ARG.
 * Host buffers; synchronous. */
int dl_trace_closest_wavefront(dl_scene* scene, const float* rays, int64_t n,
                               int32_t* prim_id, float* t, float* u, float* v);
int dl_trace_any_wavefront(dl_scene* scene, const float* rays, int64_t n, uint8_t* occluded);

/* -------------------------------------------------------------- rendering */

enum dl_filter {
    DL_FILTER_GAUSSIAN = 0,  /* src/tracer/rfilter/rfilter.cpp:13-35, radius 2, stddev 0.5 */
    DL_FILTER_BOX = 1        /* src/tracer/rfilter/rfilter.cpp:83-96, radius 0.5 */
};

enum dl_render_flags {
    /* Point light with the receiver cosine and MIS weight 1 (OptiX form,
     * include/optix/light/point.h:15-42, src/optix/cuda/hitgroup_pgs.cu:99).
     * Off: the reference CPU form (no cosine, power-heuristic weight,
     * src/tracer/emitter/point.cpp:17-33, src/tracer/integrator/path.cpp:53). */
    DL_RENDER_FIX_POINT_LIGHT = 1u << 0,
    /* Pick the NEE emitter through an alias table in proportion to an
     * estimate of its power -- area: pi * area * max(radiance); point:
     * 4 pi * max(intensity); envmap: pi * R^2 * integral of max(radiance) over
     * the sphere, R the radius of the scene's bounding sphere -- instead of
     * uniformly (src/tracer/scene/scene.cpp:148-163).  The pick probability
     * replaces 1/N in the NEE weight and in the MIS weights of emitter hits. */
    DL_RENDER_POWER_LIGHT_PICK = 1u << 1,
    /* The "normals" integrator (NormalIntegrator::Li,
     * src/tracer/integrator/normal.cpp:8-20): each sample is the componentwise
     * absolute value of the shading normal at the camera ray's first hit, 0
     * when it misses.  Set in the scene's default options by an XML
     * <integrator type="normals"/>.  Not available for guided renders. */
    DL_RENDER_NORMALS = 1u << 2
};

/* Render options.  Reference: PathIntegrator (src/tracer/integrator/path.cpp),
 * Independent sampler (src/tracer/sampler/independent.cpp) and the
 * CPURenderer sample loop (src/tracer/backend/cpu_renderer.cpp:22-55). */
typedef struct dl_render_opts {
    int32_t spp;             /* samples per pixel */
    int32_t max_depth;       /* <= 0: unbounded, as the reference; else at most
                                max_depth scattering events per path */
    int32_t rr_depth;        /* Russian roulette when depth > rr_depth (reference: 3) */
    int32_t filter;          /* dl_filter */
    uint64_t seed;           /* pcg32 seed of every path stream */
    uint32_t flags;          /* dl_render_flags */
    int32_t spp_offset;      /* index of the first sample (disjoint ranges for replicas) */
    int64_t max_paths_in_flight; /* wavefront pool size; 0 = automatic */
} dl_render_opts;

/* Default options for a scene (spp / filter from XML when loaded from XML;
 * otherwise spp 1, unbounded depth, rr_depth 3, Gaussian filter, seed 0). */
int dl_scene_default_opts(const dl_scene* scene, dl_render_opts* opts);

/* Render the scene's camera view.  rgb_out: height x width x 3 floats
 * (row 0 = top image row, as the reference's bitmap), each pixel the
 * filter-weighted mean of its samples (ImageBlock::put / toBitmap,
 * src/core/bitmap/block.cpp:58-113).  Host buffer. */
int dl_render(dl_scene* scene, const dl_render_opts* opts, float* rgb_out);

/* Same render, but returns the raw film: (height + 2b) x (width + 2b) x 4
 * floats (weighted RGB sums and weight sum, b = filter border: 2 for the
 * Gaussian, 0 for the box).  Films of disjoint sample ranges add up. */
int dl_render_film(dl_scene* scene, const dl_render_opts* opts, float* film_out);

/* Device form of dl_render_film: film written to a device buffer on the
 * context stream; the call returns without synchronising. */
int dl_render_film_device(dl_scene* scene, const dl_render_opts* opts, float* d_film);

/* --------------------------------------------------------------- images */

enum dl_image_format {
    DL_IMAGE_PNG = 0,  /* Bitmap::savePNG (src/core/bitmap/bitmap.cpp:190-214): sRGB
                          (Color3f::toSRGB, include/core/bitmap/color.h:76-87), x255,
                          clamped to [0, 255], truncated to 8 bits */
    DL_IMAGE_EXR = 1,  /* Bitmap::saveEXR (bitmap.cpp:157-188): float R, G, B; written
                          uncompressed */
    DL_IMAGE_PFM = 2   /* linear floats, little endian, rows bottom to top */
};

/* Write an RGB image (height x width x 3 floats, row 0 = top, as dl_render
 * returns it) to `path` (the full file name; the reference appends ".png" /
 * ".exr" itself).  Host only: needs no context or GPU.  Messages of failed
 * calls: dl_last_error(NULL). */
int dl_image_write(const char* path, int32_t width, int32_t height, const float* rgb, int32_t format);

/* Read a PNG (8-bit grey / grey + alpha / RGB / RGBA / palette, not
 * interlaced; values = bytes / 255, alpha dropped) or PFM image as RGB
 * floats, row 0 = the image's top row.  With rgb NULL only width and height
 * are returned; then call again with capacity >= width * height * 3.  The
 * reference reads bitmaps with stb_image / OpenEXR
 * (src/core/bitmap/bitmap.cpp:33-152); host only. */
int dl_image_read(const char* path, int32_t* width, int32_t* height, float* rgb, int64_t capacity);

/* Radiance of individual camera paths, the reference's
 * Integrator::Li(scene, sampler, ray) (include/tracer/integrator.h:38) for
 * the paths (x, y, s) given as n triples: pixel x, pixel y, sample index s.
 * Each path draws its pixel sample, aperture sample and all bounce samples
 * from its own pcg32 stream, exactly as dl_render does for that (x, y, s).
 * L_out: n x 3 radiance; pos_out: n x 2 film position of the sample (may be
 * NULL).  Host buffers. */
int dl_li(dl_scene* scene, const dl_render_opts* opts, int64_t n,
          const int32_t* xys, float* L_out, float* pos_out);

/* Allocation-free form of dl_li, with no counterpart in the reference.  For
 * callers that may not allocate device memory while rendering (an engine
 * that owns all device memory after start-up, a loop with a fixed memory
 * budget, a thread that may not block on the allocator): the path state
 * lives in one fixed array of 16384 path slots (3.75 MiB) compiled into the
 * library, present on every GPU that loads it until the process exits.
 * d_xys (n x 3 int32), d_L (n x 3 float) and d_pos (n x 2 float) are device
 * pointers supplied by the caller.  opts->max_paths_in_flight must be 0
 * (whole pool) or at most 16384, else DL_ERR_INVALID_ARG.  The first call on
 * a device resolves the array's address, so make it before any stream
 * capture.  All calls, from every context on the device, share the array:
 * calls whose work overlaps on the GPU race, so the caller serialises them.
 * A synchronous call on the context stream: it returns after the paths
 * finish, with the status codes and messages of dl_li for the same faults. */
int dl_li_static(dl_scene* scene, const dl_render_opts* opts, int64_t n,
                 const int32_t* d_xys, float* d_L, float* d_pos);

/* BSDF::eval, BSDF::pdf and BSDF::sample (include/tracer/bsdf.h:62-104;
 * for aniso_ggx the OptiX callables of src/optix/cuda/material/
 * aniso_ggx.cu:37-121) of one material (its constant parameters; textures
 * are not used) on n queries, evaluated on the GPU by the device code the
 * material kernels run.  wi, wo: n x 3 local directions (eval and pdf of
 * (wi, wo) in solid-angle measure); smp: n x 3 uniform numbers for sample(wi):
 * the 2D sample, then the lobe coin that only aniso_ggx draws
 * (aniso_ggx.cu:104-108).  Outputs: eval n x 3, pdf n, sampled wo n x 3,
 * sample weight n x 3, eta n, measure n (0 unknown, 1 solid angle,
 * 2 discrete).  Host buffers; synchronous. */
int dl_bsdf_query(dl_context* ctx, const dl_material_desc* material, int64_t n,
                  const float* wi, const float* wo, const float* smp,
                  float* eval, float* pdf, float* s_wo, float* s_weight, float* s_eta,
                  int32_t* s_measure);

/* The scene's environment emitter on the GPU: Envmap::sampleDirection from
 * three uniform numbers xi (n x 3) at shading normals nrm (n x 3) --
 * direction s_dir, solid-angle pdf s_pdf, and cos * radiance / pdf s_value --
 * and Envmap::pdfDirection / Envmap::eval of the directions dirs (n x 3)
 * (include/optix/light/envmap.h:25-94).  DL_ERR_INVALID_ARG when the scene
 * has no envmap.  Host buffers; synchronous. */
int dl_scene_env_query(dl_scene* scene, int64_t n, const float* xi, const float* nrm,
                       const float* dirs, float* s_dir, float* s_pdf, float* s_value,
                       float* pdf, float* value);

/* Scene::sampleEmitterDirection (src/tracer/scene/scene.cpp:139-170)
 * without its visibility test, on the GPU, by the code the material kernels
 * run: at points pts with shading normals nrm (n x 3 each) and 2D samples
 * smp (n x 2), the emitter picked uniformly (the reference) or, with
 * DL_RENDER_POWER_LIGHT_PICK in flags, by the power alias table; outputs the
 * direction d (n x 3), distance, solid-angle pdf times the pick probability,
 * the unoccluded spectrum / pdf (n x 3) and the picked emitter index.  An
 * envmap pick draws its three numbers from a per-query pcg32.  Host
 * buffers; synchronous. */
int dl_scene_emitter_sample(dl_scene* scene, uint32_t flags, int64_t n, const float* pts,
                            const float* nrm, const float* smp, float* d, float* dist, float* pdf,
                            float* spec, int32_t* light);

/* Measurement aid, no counterpart in the reference: the device's L2 -> SM
 * read bandwidth in GB/s, from a kernel that streams an L2-resident buffer
 * of `bytes` (1 MiB .. 4 GiB; 64 MiB fits the GB300's L2) `passes` times
 * with L2-only loads after one warm-up pass.  The traversal kernels' node
 * and triangle fetches are bounded by it when the BVH stays in L2. */
int dl_measure_l2_read_bandwidth(dl_context* ctx, int64_t bytes, int32_t passes, double* gbs);

/* ----------------------------------------------------------------- batches */

/* One request of a batch: a scene of the context, its render options and at
 * least one output -- `rgb` (host, height x width x 3, as dl_render) and/or
 * `film_device` (device film, as dl_render_film_device). */
typedef struct dl_request {
    dl_scene* scene;
    dl_render_opts opts;
    float* rgb;
    float* film_device;
    const dl_camera_desc* camera;  /* NULL: the scene's camera; else this one
                                      (its resolution sizes the outputs) */
} dl_request;

/* Render many requests -- of different scenes, resolutions and sample
 * counts -- in one wavefront: their paths share the path pool, the
 * material-sorted queues and the captured iteration graph, each path
 * carrying its request; every pass renders a slice of every unfinished
 * request's samples and gathers each slice into its request's film.  Each
 * request's image equals its dl_render image up to float summation order.
 * No reference counterpart: the reference renders one scene per process
 * (src/main.cpp, src/tracer/backend/cpu_renderer.cpp). */
int dl_render_batch(dl_context* ctx, const dl_request* reqs, int32_t n);

/* Launch shape of the wavefront renderer: path slots in flight (the pool),
 * CTAs per SM of the traversal kernels and of the shading kernels, threads
 * per CTA of the shading kernels (the miss and the material kernels),
 * wavefront iterations per captured graph launch (between queue checks). */
typedef struct dl_tune_params {
    int64_t paths_in_flight;        /* 32 .. 2^28; opts.max_paths_in_flight overrides */
    int32_t traverse_ctas_per_sm;   /* 1 .. 16 */
    int32_t shade_ctas_per_sm;      /* 1 .. 64 */
    int32_t iterations_per_graph;   /* 2, 4, 6 or 8 */
    int32_t shade_threads;          /* 64, 128 or 256; 0 = 128 */
} dl_tune_params;
int dl_context_get_tune(const dl_context* ctx, dl_tune_params* out);
int dl_context_set_tune(dl_context* ctx, const dl_tune_params* tune);

/* Autotuner: renders the requests at `trial_spp` samples per pixel each (0:
 * an eighth of each request's spp, at least 1) under candidate launch shapes
 * -- a coordinate search over the pool size, then the traversal and shading
 * grid sizes, the shading block size, then the graph length -- times each
 * on the GPU, and keeps the
 * fastest on the context.  `out` (may be NULL) receives it; `trials` (may be
 * NULL) the number of shapes timed.  Outputs of the requests are not written. */
int dl_autotune(dl_context* ctx, const dl_request* reqs, int32_t n, int32_t trial_spp, dl_tune_params* out,
                int32_t* trials);

/* ------------------------------------------------------- learned guiding */

/* A learned proposal for path guiding: an MLP on (position, normal) whose
 * output is a mixture of 8 von Mises-Fisher lobes over incident directions,
 * trained online on the renderer's own radiance samples and used as one
 * extra technique in one-sample MIS with BSDF sampling (the estimator stays
 * unbiased; BSDF + NEE remains the fallback).  No reference counterpart.
 *
 * Network: encoding sin/cos(2^(k-3) pi x), k < 12, of the 6 inputs (144
 * features) -> 64 ReLU -> 64 ReLU -> 40 outputs = per lobe (mean direction
 * m (3, normalised), log kappa (clamped to [-3, 8]), weight logit (softmax)).
 * FP16 weights and activations, FP32 accumulation, on the tensor cores.
 * Parameters (DL_GUIDE_PARAMS floats): W1 [64][144], b1 [64], W2 [64][64],
 * b2 [64], W3 [48][64] (rows 40..47 zero), b3 [48] (40..47 zero). */
#define DL_GUIDE_PARAMS 16560
typedef struct dl_guide dl_guide;
typedef struct dl_guide_config {
    float learning_rate;     /* Adam step size (2e-3) */
    float guide_fraction;    /* probability of sampling the learned proposal at a guided vertex (0.5) */
    int32_t batch;           /* training records per Adam step (131072) */
    int32_t steps_per_pass;  /* Adam steps after each pass of dl_render_guided (16) */
    int32_t max_guided_depth; /* vertices at this depth or deeper sample the BSDF alone (6) */
    int32_t reserved;
    uint64_t seed;           /* initial weights */
} dl_guide_config;
int dl_guide_default_config(dl_guide_config* cfg);
int dl_guide_create(dl_context* ctx, const dl_guide_config* cfg, dl_guide** out);
int dl_guide_destroy(dl_guide* guide);
int dl_guide_get_params(const dl_guide* guide, float* params);
int dl_guide_set_params(dl_guide* guide, const float* params);
/* Network outputs (n x 40) for inputs (n x 6: position in [0,1]^3, normal). */
int dl_guide_forward(dl_guide* guide, int64_t n, const float* inputs, float* outputs);
/* Training records, 12 floats each: position in [0,1]^3 (3), normal (3),
 * sampled direction (3), its sampling pdf, radiance estimate along it, 0.
 * Loss: -(1/n) sum min((L/p) / mean(L/p), 20) log q(direction).  dl_guide_gradient
 * returns the gradient of that loss (DL_GUIDE_PARAMS floats) and the loss
 * without updating; dl_guide_train runs `steps` Adam steps on the batch. */
int dl_guide_gradient(dl_guide* guide, int64_t n, const float* records, float* grad, float* loss);
int dl_guide_train(dl_guide* guide, int64_t n, const float* records, int32_t steps, float* loss);

/* Progressive guided render (as dl_render, image to host): passes of 1, 1,
 * 2, 4, ... samples per pixel.  Guided vertices are those on diffuse,
 * Beckmann and GGX surfaces shallower than max_guided_depth.  With `train`
 * set, a hashed subset of each pass's guided vertices -- about batch x
 * steps_per_pass of them, spread over the whole image -- become training
 * records (radiance gathered later on the path is credited to the two most
 * recent ones) and the guide takes steps_per_pass Adam steps on interleaved
 * subsets of them before the next pass.  With `train` 0 the network is
 * frozen.  All samples add to one film. */
int dl_render_guided(dl_scene* scene, const dl_render_opts* opts, dl_guide* guide, int32_t train, float* rgb_out);

/* --------------------------------------------------------------- statistics */

typedef struct dl_stats {
    int64_t camera_rays;       /* paths started */
    int64_t extension_rays;    /* closest-hit rays traced (camera rays included) */
    int64_t shadow_rays;       /* any-hit rays traced */
    int64_t invalid_samples;   /* samples dropped by the film (NaN/Inf/negative) */
    int64_t iterations;        /* wavefront iterations of the last render */
    double render_ms;          /* device time of the last render */
    double trace_ms;           /* device time of the last dl_trace_* call */
    /* Per-kernel device time of the last render, summed over its launches
     * (CUDA events on the context stream; filled only while kernel timing is
     * enabled, see dl_context_set_kernel_timing). */
    double extend_ms;          /* closest-hit traversal */
    double shadow_ms;          /* any-hit traversal */
    double shade_ms;           /* the material kernels (emitter hit, RR, NEE, BSDF sampling) */
    double retire_ms;          /* the miss kernel (envmap, sample store, new camera paths) */
    int64_t kernel_launches;   /* kernels launched by the last render */
    int64_t guide_records;     /* training records written by the last guided render */
    double guide_train_ms;     /* device time of the last training round of the last guided
                                  render (rounds overlap the next pass's rendering) */
    double guide_ms;           /* device time of the network kernels of the last
                                  dl_guide_forward / dl_guide_gradient call */
} dl_stats;

/* Enable (1) or disable (0) per-kernel event timing on a context. */
int dl_context_set_kernel_timing(dl_context* ctx, int enabled);

/* Counters of the last dl_render* / dl_li / dl_trace_* call on ctx. */
int dl_stats_get(const dl_context* ctx, dl_stats* stats);

/* Measurement aid (not for timing): repeats a render with per-ray traversal
 * counters enabled and reports the BVH node visits and triangle tests of its
 * extension and shadow rays.  No reference counterpart. */
typedef struct dl_traversal_counts {
    int64_t extension_rays;
    int64_t shadow_rays;
    int64_t extension_node_visits;     /* BVH nodes fetched by closest-hit rays */
    int64_t extension_triangle_tests;  /* triangles tested by closest-hit rays */
    int64_t shadow_node_visits;
    int64_t shadow_triangle_tests;
} dl_traversal_counts;
int dl_render_traversal_counts(dl_scene* scene, const dl_render_opts* opts, dl_traversal_counts* out);

#ifdef __cplusplus
}
#endif

#endif /* DRAWLAB_H */
