/*
 * oracle.h -- CPU restatement of the xuxmin/DrawLab path-tracer hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Tests, __graft_entry__.smoke() and bench.py's
 * CPU baseline call it as the oracle; the product never links it.
 *
 * Scene input is the dl_*_desc arrays of include/drawlab.h.  Every entry
 * point restates the reference function named beside it (paths relative to
 * the reference project root).
 */
#ifndef DRAWLAB_ORACLE_H
#define DRAWLAB_ORACLE_H

#include <stdint.h>

#include "drawlab.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Build the scene and its octree (Scene::addChild/activate, OCTree::build). */
void* orc_scene_create(const dl_mesh_desc* meshes, int32_t num_meshes,
                       const dl_material_desc* materials, int32_t num_materials,
                       const dl_light_desc* lights, int32_t num_lights,
                       const dl_camera_desc* camera, int32_t filter);
void orc_scene_destroy(void* scene);
const char* orc_last_error(void);

/* OCTree closest hit / any hit (src/tracer/accel/octree.cpp:53-133). */
int orc_trace_closest(void* scene, const float* rays, int64_t n, int32_t* prim, float* t,
                      float* u, float* v, int32_t threads);
int orc_trace_any(void* scene, const float* rays, int64_t n, uint8_t* occluded,
                  int32_t threads);

/* The reference CPU render: spiral 32x32 blocks, one pcg32 stream per block
 * seeded with the block offset (src/tracer/backend/cpu_renderer.cpp:22-135).
 * max_blocks > 0 renders only the first max_blocks blocks of the spiral. */
int orc_render_blocks(void* scene, const dl_render_opts* opts, int32_t threads,
                      int32_t max_blocks, float* rgb_out, float* film_out, double* seconds);

/* The block renderer over the blocks at the given positions of the spiral
 * order (each with its own per-block pcg32); orc_num_blocks is the number of
 * 32x32 blocks of the image.  Returns nonzero for an index out of range. */
int orc_render_block_subset(void* scene, const dl_render_opts* opts, int32_t threads, int32_t n,
                            const int32_t* spiral_index, float* rgb_out, float* film_out, double* seconds);
int orc_num_blocks(void* scene);

/* Per-path streams (the GPU renderer's sampling): every (x, y, s) path seeds
 * its own pcg32.  Film and rgb as dl_render_film / dl_render. */
int orc_render_paths(void* scene, const dl_render_opts* opts, int32_t threads,
                     float* rgb_out, float* film_out, double* seconds);

/* Li of explicit (x, y, s) paths (as dl_li). */
int orc_li(void* scene, const dl_render_opts* opts, int64_t n, const int32_t* xys,
           float* L_out, float* pos_out, int32_t threads);

/* BSDF::eval / pdf / sample on given local directions (see ref_bsdf_query);
 * smp holds three uniform numbers per query: the 2D sample and the lobe
 * coin that only aniso_ggx draws (aniso_ggx.cu:104-108). */
int orc_bsdf_query(const dl_material_desc* m, int64_t n, const float* wi, const float* wo,
                   const float* smp, float* eval, float* pdf, float* s_wo, float* s_w,
                   float* s_eta, int32_t* s_measure);

/* Frame(n) (include/core/math/frame.h:104-123). */
int orc_frame(int64_t n, const float* nrm, float* t, float* b);

/* Scene::sampleEmitterDirection at given points (see ref_emitter_sample). */
int orc_emitter_sample(void* scene, const dl_render_opts* opts, int64_t n, const float* pts,
                       const float* nrm, const float* smp, float* d, float* dist, float* pdf,
                       float* spec);

/* The envmap's alias table and pdf (src/tracer/emitter/envmap.cpp:59-141),
 * env_width x env_height entries each.  Returns nonzero without an envmap. */
int orc_env_tables(void* scene, float* q, uint32_t* alias, float* pdf);

/* The oracle's pcg32: n outputs of seed(initstate, initseq) as nextUInt and
 * as nextFloat (independent.cpp:31-45 with the wjakob/pcg32 interface). */
int orc_pcg32(uint64_t initstate, uint64_t initseq, int32_t n, uint32_t* out, float* out_float);

/* Envmap::sampleDirection from three numbers xi at shading normals nrm, and
 * pdfDirection / eval of dirs (include/optix/light/envmap.h:25-94).  Returns
 * nonzero without an envmap. */
int orc_env_query(void* scene, int64_t n, const float* xi, const float* nrm, const float* dirs,
                  float* s_dir, float* s_pdf, float* s_val, float* pdf, float* val);

/* __miss__radiance (src/optix/cuda/miss.cu:11-49): radiance of rays leaving
 * along dirs after a bounce of depth[i] (0: camera ray) whose BSDF sample had
 * pdf bsdf_pdf[i] and diffuse flag is_diffuse[i]. */
int orc_env_miss(void* scene, const dl_render_opts* opts, int64_t n, const float* dirs,
                 const int32_t* depth, const float* bsdf_pdf, const uint8_t* is_diffuse, float* out);

/* Camera ray through film positions film (n x 2, pixel units). */
int orc_camera_ray(void* scene, int64_t n, const float* film, float* o, float* d);

/* Hit record of global triangle prim[i] at barycentrics bary[i]: shading
 * normal, geometric normal, shading tangent (0: none) and texture
 * coordinates (shader_common.h:21-143 for maps and texcoords). */
int orc_hit_data(void* scene, int64_t n, const int32_t* prim, const float* bary, float* sn,
                 float* gn, float* st, float* tuv);

#ifdef __cplusplus
}
#endif

#endif
