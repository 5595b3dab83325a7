// Device-visible scene layout (plain structs shared by host and device code).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace dl {

// ------------------------------------------------------------------ layout
constexpr int32_t kEmptyChild = 0x7fffffff;
constexpr int kStackSize = 64;
constexpr float kRayEps = 1e-4f;   // M_EPSILON, include/core/math/math.h:14
constexpr float kPiF = 3.14159265358979323846f;
constexpr float kInvPiF = 0.31830988618379067154f;
constexpr float kInvTwoPiF = 0.15915494309189533577f;

enum MatType { MAT_DIFFUSE = 0, MAT_MIRROR = 1, MAT_DIELECTRIC = 2, MAT_MICROFACET = 3, MAT_ANISO_GGX = 4 };
enum LightType { LIGHT_AREA = 0, LIGHT_POINT = 1, LIGHT_ENVMAP = 2 };

// texture slots of a material (dl_material_desc's *_texture fields)
enum TexSlot { TEX_ALBEDO = 0, TEX_SPECULAR = 1, TEX_ALPHA = 2, TEX_NORMAL = 3, TEX_TANGENT = 4, kTexSlots = 5 };

struct DevMaterial {
    int type;
    float albedo[3];
    float specular[3];
    float ax, ay;
    float int_ior, ext_ior;
    float ks;          // microfacet: 1 - max(kd)
    int tex[kTexSlots];  // texture index per slot, -1 = none
    int has_tex;         // any slot set
};

struct DevTexture {
    const float4* texels;  // rgb + pad, row k at t = (k + 0.5) / h
    int w, h;
};

struct DevMesh {
    int material;
    int light;         // emitter index or -1
    int has_normals;
    int has_texcoords;
};

struct DevLight {
    int type;
    int mesh;
    int tri_begin;     // area: first entry in emit_tris (6 float4 per triangle)
    int tri_count;
    int cdf_begin;     // area: first entry in emit_cdf (tri_count + 1 floats)
    int has_normals;
    float pA;          // area: 1 / total area (DiscretePDF normalisation)
    float radiance[3];
    float position[3];
};

struct DevCamera {
    int w, h;
    float eye[3], U[3], V[3], W[3];  // virtual (opencv: eye)
    float inv_w, inv_h;
    int type;                        // dl_camera_type
    float S[16];                     // perspective: sample-to-camera, row-major
    float T[16];                     // perspective: camera-to-world; opencv: inverse extrinsic
    float far_clip;                  // perspective
    float fx, fy, cx, cy;            // opencv
};

struct DevScene {
    const float4* __restrict__ nodes;     // 4 float4 per node
    const float4* __restrict__ tris;      // 3 float4 per triangle (leaf order)
    const int4* __restrict__ tri_vidx;    // per leaf-order triangle: vertex ids + mesh id
    const float4* __restrict__ normals;   // per vertex (global index), w unused
    const DevMesh* __restrict__ meshes;
    const DevMaterial* __restrict__ materials;
    const DevLight* __restrict__ lights;
    const float4* __restrict__ emit_tris;
    const float* __restrict__ emit_cdf;
    const DevTexture* __restrict__ textures;
    const float2* __restrict__ texcoords;  // per vertex (global index)
    int num_tris;
    int num_nodes;
    int num_lights;
    DevCamera cam;
    // environment light (env_light < 0: none).  Texels rgb+pad, row 0 at the
    // +y pole; per texel {alias probability q, alias index, pdf, 0}.
    const float4* __restrict__ env_tex;
    const float4* __restrict__ env_accel;
    // power-proportional emitter pick: per light {alias q, alias index, pick
    // probability, 0}
    const float4* __restrict__ light_pick;
    // bounds of every vertex: position -> [0, 1]^3 for the guiding network
    float bb_lo[3];
    float bb_inv_ext[3];
    int env_light;
    int env_w, env_h;
    int env_visual;
    float env_scale;
    float env_bg[3];
};

}  // namespace dl
