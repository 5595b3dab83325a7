// Reference harness, OptiX half (TEST INFRASTRUCTURE ONLY; never shipped).
//
// The reference implements its GGX / anisotropic GGX material, environment
// map emitter, environment miss shading, OpenCV camera and texture lookups
// only in its OptiX backend.  This file compiles that code -- the
// reference's own headers and .cu shader sources, where they lie -- as host
// C++ (g++ with __CUDACC__ defined, so that its SUTIL_HOSTDEVICE members are
// compiled; the CUDA qualifiers become ignored attributes) against the
// stand-ins of oracle/ref_shim_optix: CUDA's vector types, a host model of
// tex2D<float4> and host versions of the OptiX ray / hit queries.  The C
// functions below drive the reference code and are what
// tests/golden/make_golden.py records as golden vectors:
//
//   refx_ggx_*          src/optix/cuda/material/aniso_ggx.cu:9-121 and
//                       include/optix/math/wrap.h:54-77
//   refx_env_*          include/optix/light/envmap.h:25-94
//   refx_env_miss       src/optix/cuda/miss.cu:11-49
//   refx_opencv_ray     include/optix/camera/opencv.h:24-47
//   refx_hit_data       src/optix/cuda/shader_common.h:21-143 (texcoords,
//                       normal and tangent maps, shading frame inputs)
//   refx_texture_*      the host model of the reference's CUDA textures
//                       (linear filtering, wrap addressing, normalized
//                       coordinates: src/optix/host/cuda_texture.cpp:57-84)
#include <cuda_runtime.h>
#include <optix.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "optix/camera/opencv.h"
#include "optix/light/envmap.h"
#include "optix/math/onb.h"
#include "optix/math/vec_math.h"
#include "optix/math/wrap.h"
#include "material/aniso_ggx.cu"
#include "miss.cu"

namespace optix {
extern "C" {
Params params;
}
}  // namespace optix

// ------------------------------------------------------------- host model
namespace refshim {
OptixState g_optix;
bool g_quantised_weights = false;

namespace {
std::vector<HostTexture> g_textures;
std::vector<std::vector<float4>> g_texels;
}  // namespace

HostTexture* texture_slot(cudaTextureObject_t obj) { return &g_textures.at((size_t)obj - 1); }

// Linear filtering of a 2D texture with normalized coordinates and wrap
// addressing, as the CUDA C Programming Guide's texture-fetching appendix
// states it: x -> frac(x) * W - 0.5, i = floor, alpha = frac, texels i and
// i + 1 taken modulo W (rows alike), the four texels blended with weights
// (1 - a)(1 - b), a(1 - b), (1 - a)b, ab.  With g_quantised_weights the
// fractions are rounded to the texture unit's 8 fractional bits.
float4 tex2d_linear_wrap(const HostTexture& t, float u, float v) {
    u = u - std::floor(u);
    v = v - std::floor(v);
    float x = u * (float)t.width - 0.5f;
    float y = v * (float)t.height - 0.5f;
    float fx = std::floor(x), fy = std::floor(y);
    float ax = x - fx, ay = y - fy;
    if (g_quantised_weights) {
        ax = std::nearbyint(ax * 256.0f) / 256.0f;
        ay = std::nearbyint(ay * 256.0f) / 256.0f;
    }
    int x0 = (int)fx, y0 = (int)fy;
    int x1 = x0 + 1, y1 = y0 + 1;
    auto wrap = [](int i, int n) { return ((i % n) + n) % n; };
    x0 = wrap(x0, t.width);
    x1 = wrap(x1, t.width);
    y0 = wrap(y0, t.height);
    y1 = wrap(y1, t.height);
    const float4 t00 = t.texels[(size_t)y0 * t.width + x0], t10 = t.texels[(size_t)y0 * t.width + x1];
    const float4 t01 = t.texels[(size_t)y1 * t.width + x0], t11 = t.texels[(size_t)y1 * t.width + x1];
    const float bx = 1.f - ax, by = 1.f - ay;
    const float w00 = bx * by, w10 = ax * by, w01 = bx * ay, w11 = ax * ay;
    return make_float4(t00.x * w00 + t10.x * w10 + t01.x * w01 + t11.x * w11,
                       t00.y * w00 + t10.y * w10 + t01.y * w01 + t11.y * w11,
                       t00.z * w00 + t10.z * w10 + t01.z * w01 + t11.z * w11,
                       t00.w * w00 + t10.w * w10 + t01.w * w01 + t11.w * w11);
}
}  // namespace refshim

namespace {
float3 ld3(const float* p) { return make_float3(p[0], p[1], p[2]); }
void st3(float* p, float3 v) {
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}
// The reference's rnd(): the numbers the shader code will draw from a copy
// of the seed, so the golden files can record them.  peek3 takes three in
// sequence (statements in order: aniso_ggx.cu:100-108); the two forms
// below repeat the shaders' own expressions, make_float3(rnd(seed),
// rnd(seed), rnd(seed)) (envmap.h:35) and make_float2(x + rnd(seed), y +
// rnd(seed)) (opencv.h:39), whose argument evaluation order C++ leaves to
// the compiler: repeating the expression records the order the compiler
// chose for this harness.
float3 peek3(unsigned int seed) {
    float a = rnd(seed);
    float b = rnd(seed);
    float c = rnd(seed);
    return make_float3(a, b, c);
}
float3 peek_env_xi(unsigned int seed) { return make_float3(rnd(seed), rnd(seed), rnd(seed)); }
float2 peek_jitter(unsigned int seed) {
    const float x = 0.f, y = 0.f;
    return make_float2(x + rnd(seed), y + rnd(seed));
}

optix::Material ggx_material(const float* pd, const float* ps, float ax, float ay, cudaTextureObject_t pd_tex,
                             cudaTextureObject_t ps_tex, cudaTextureObject_t axay_tex) {
    optix::Material m;
    std::memset((void*)&m, 0, sizeof(m));
    m.type = optix::Material::ANISOGGX;
    m.aniso_ggx.pd = ld3(pd);
    m.aniso_ggx.ps = ld3(ps);
    m.aniso_ggx.axay = make_float2(ax, ay);
    m.aniso_ggx.pd_tex = pd_tex;
    m.aniso_ggx.ps_tex = ps_tex;
    m.aniso_ggx.axay_tex = axay_tex;
    m.normal_tex = 0;
    m.tangent_tex = 0;
    m.is_tangent_space = false;
    m.is_diffuse = true;
    m.is_hide = false;
    return m;
}

optix::Envmap g_env;
std::vector<optix::EnvAccel> g_env_accel;
}  // namespace

extern "C" {

// ---------------------------------------------------------------- textures
// Register an RGBA float texture (height x width x 4, row 0 = v in [0, 1/H))
// in the host model; returns its object id (> 0).
unsigned long long refx_texture_create(int32_t width, int32_t height, const float* rgba) {
    using namespace refshim;
    g_texels.emplace_back((size_t)width * height);
    std::memcpy(g_texels.back().data(), rgba, sizeof(float4) * (size_t)width * height);
    HostTexture t;
    t.width = width;
    t.height = height;
    t.texels = g_texels.back().data();
    g_textures.push_back(t);
    // earlier entries' texel pointers stay valid: each vector owns its heap block
    return (unsigned long long)g_textures.size();
}

void refx_texture_reset(void) {
    refshim::g_textures.clear();
    refshim::g_texels.clear();
}

void refx_set_quantised_weights(int32_t on) { refshim::g_quantised_weights = on != 0; }

void refx_texture_lookup(unsigned long long obj, int64_t n, const float* uv, float* out) {
    for (int64_t i = 0; i < n; i++) {
        float4 r = tex2D<float4>(obj, uv[2 * i], uv[2 * i + 1]);
        out[4 * i] = r.x;
        out[4 * i + 1] = r.y;
        out[4 * i + 2] = r.z;
        out[4 * i + 3] = r.w;
    }
}

// ------------------------------------------------------------ aniso_ggx
// eval / pdf (aniso_ggx.cu:37-75) of (wi, wo) and sample (aniso_ggx.cu:
// 89-121) of wi with the shader's own rnd() stream from seeds[i]; xi
// receives the three numbers that stream yields (z1, z2, lobe coin).
// Texture ids of 0 mean constant pd / ps / axay; uv (n x 2) is the hit's
// texture coordinate.
void refx_ggx(int64_t n, const float* pd, const float* ps, float ax, float ay, unsigned long long pd_tex,
              unsigned long long ps_tex, unsigned long long axay_tex, const float* uv, const float* wi,
              const float* wo, const uint32_t* seeds, float* eval, float* pdf, float* xi, float* s_wo,
              float* s_w) {
    using namespace optix;
    const Material m = ggx_material(pd, ps, ax, ay, pd_tex, ps_tex, axay_tex);
    for (int64_t i = 0; i < n; i++) {
        Intersection its;
        std::memset((void*)&its, 0, sizeof(its));
        its.uv = uv ? make_float2(uv[2 * i], uv[2 * i + 1]) : make_float2(0.f, 0.f);
        BSDFQueryRecord q(its, ld3(wi + 3 * i), ld3(wo + 3 * i), ESolidAngle);
        st3(eval + 3 * i, __direct_callable__anisoggx_eval(m, q));
        pdf[i] = __direct_callable__anisoggx_pdf(m, q);
        unsigned int seed = seeds[i];
        st3(xi + 3 * i, peek3(seed));
        BSDFQueryRecord s(its, ld3(wi + 3 * i));
        s.wo = make_float3(0.f, 0.f, 0.f);
        float3 w = __direct_callable__anisoggx_sample(m, seed, s);
        st3(s_wo + 3 * i, s.wo);
        st3(s_w + 3 * i, w);
    }
}

// Wrap::squareToGGX / squareToGGXPdf (wrap.h:54-77) on given samples and
// half vectors.
void refx_square_to_ggx(int64_t n, float ax, float ay, const float* smp, const float* m, float* wh, float* d) {
    for (int64_t i = 0; i < n; i++) {
        st3(wh + 3 * i, optix::Wrap::squareToGGX(make_float2(smp[2 * i], smp[2 * i + 1]), make_float2(ax, ay)));
        d[i] = optix::Wrap::squareToGGXPdf(ld3(m + 3 * i), make_float2(ax, ay));
    }
}

// ------------------------------------------------------------------ envmap
// The Envmap light of envmap.h with a given alias table (q, alias, pdf per
// texel, row-major from the +y pole) and radiance texture (a texture id of
// the host model, the same row order).
void refx_env_set(int32_t width, int32_t height, unsigned long long tex, const float* q, const uint32_t* alias,
                  const float* pdf, float scale, int32_t visual) {
    g_env_accel.resize((size_t)width * height);
    for (size_t i = 0; i < g_env_accel.size(); i++) {
        g_env_accel[i].q = q[i];
        g_env_accel[i].alias = alias[i];
        g_env_accel[i].pdf = pdf[i];
    }
    std::memset((void*)&g_env, 0, sizeof(g_env));
    g_env.env_tex = tex;
    g_env.env_accel = g_env_accel.data();
    g_env.env_size = make_int2(width, height);
    g_env.visual = visual != 0;
    g_env.scale = scale;
}

// Envmap::sampleDirection (envmap.h:33-76) at shading points p with normals
// sn, drawing its three numbers from rnd(seeds[i]) (recorded in xi as the
// shader uses them: xi.x picks the texel, xi.y is the alias coin, xi.z the
// position in the texel's cos(theta) range).
void refx_env_sample(int64_t n, const float* p, const float* sn, const uint32_t* seeds, float* xi, float* d,
                     float* pdf, float* ret) {
    using namespace optix;
    for (int64_t i = 0; i < n; i++) {
        Intersection its;
        std::memset((void*)&its, 0, sizeof(its));
        its.p = ld3(p + 3 * i);
        its.sn = ld3(sn + 3 * i);
        unsigned int seed = seeds[i];
        st3(xi + 3 * i, peek_env_xi(seed));
        LightSampleRecord rec;
        std::memset((void*)&rec, 0, sizeof(rec));
        float3 r = g_env.sampleDirection(its, seed, rec);
        st3(d + 3 * i, rec.d);
        pdf[i] = rec.pdf;
        st3(ret + 3 * i, r);
    }
}

// Envmap::pdfDirection, eval and environment_coords (envmap.h:25-31,78-92).
void refx_env_query(int64_t n, const float* d, float* pdf, float* val, float* uv) {
    using namespace optix;
    for (int64_t i = 0; i < n; i++) {
        LightSampleRecord rec;
        std::memset((void*)&rec, 0, sizeof(rec));
        rec.d = ld3(d + 3 * i);
        pdf[i] = g_env.pdfDirection(rec);
        Intersection its;
        std::memset((void*)&its, 0, sizeof(its));
        st3(val + 3 * i, g_env.eval(its, rec.d));
        float2 c = Envmap::environment_coords(rec.d);
        uv[2 * i] = c.x;
        uv[2 * i + 1] = c.y;
    }
}

// __miss__radiance (miss.cu:11-49) for rays leaving along d[i] after a
// bounce of depth[i] whose BSDF sample had pdf bsdf_pdf[i] and diffuse flag
// is_diffuse[i]; the scene holds num_lights lights, the envmap at env_idx.
void refx_env_miss(int64_t n, const float* d, const int32_t* depth, const float* bsdf_pdf,
                   const uint8_t* is_diffuse, int32_t num_lights, int32_t env_idx, const float* bg, float* out) {
    using namespace optix;
    std::vector<Light> lights((size_t)num_lights);
    for (int32_t k = 0; k < num_lights; k++) {
        std::memset((void*)&lights[k], 0, sizeof(Light));
        lights[k].type = Light::Type::POINT;
    }
    lights[env_idx].type = Light::Type::ENVMAP;
    lights[env_idx].envmap = g_env;
    params.light_buffer.lights = lights.data();
    params.light_buffer.light_num = num_lights;
    params.envmap_idx = env_idx;
    params.bg_color = ld3(bg);
    for (int64_t i = 0; i < n; i++) {
        RadiancePRD prd;
        std::memset((void*)&prd, 0, sizeof(prd));
        prd.depth = depth[i];
        prd.sRec.pdf = bsdf_pdf[i];
        prd.sRec.is_diffuse = is_diffuse[i] != 0;
        unsigned int p0, p1;
        packPointer(&prd, p0, p1);
        refshim::g_optix.payload0 = p0;
        refshim::g_optix.payload1 = p1;
        refshim::g_optix.ray_d = ld3(d + 3 * i);
        refshim::g_optix.ray_o = make_float3(0.f, 0.f, 0.f);
        __miss__radiance();
        st3(out + 3 * i, prd.radiance);
    }
}

// ------------------------------------------------------------------ camera
// OpencvCamera::sampleRay (opencv.h:28-46) for pixels (px, py) and sample
// indices s of an spp-sample pixel, with rnd(seeds[i]); xi receives the two
// jitter numbers as the shader adds them (x, then y).
void refx_opencv_ray(const float* inv_ext, const float* eye, float cx, float cy, float fx, float fy, int64_t n,
                     const int32_t* px, const int32_t* py, const int32_t* s, int32_t spp, const uint32_t* seeds,
                     float* xi, float* o, float* d) {
    optix::OpencvCamera cam;
    std::memcpy(cam.invExt, inv_ext, sizeof(cam.invExt));
    cam.eye = ld3(eye);
    cam.cx = cx;
    cam.cy = cy;
    cam.fx = fx;
    cam.fy = fy;
    for (int64_t i = 0; i < n; i++) {
        unsigned int seed = seeds[i];
        float2 z = peek_jitter(seed);
        xi[2 * i] = z.x;
        xi[2 * i + 1] = z.y;
        float3 ro, rd;
        cam.sampleRay(make_float2(0.f, 0.f), make_uint3((unsigned)px[i], (unsigned)py[i], 0u), seed, s[i], spp, ro,
                      rd);
        st3(o + 3 * i, ro);
        st3(d + 3 * i, rd);
    }
}

// ---------------------------------------------------------------- hit data
// getHitData (shader_common.h:21-143) for hits (prim[i], barycentrics
// bary[i]) of rays (o, d) at distance tmax[i] on one triangle mesh.  Any of
// normals / tangents / texcoords may be NULL; normal_tex / tangent_tex are
// world-space maps (texture ids, 0 = none).  Outputs: shading normal,
// geometric normal, shading tangent, texture coordinates, hit point.
void refx_hit_data(const float* positions, const float* normals, const float* tangents, const float* texcoords,
                   const int32_t* indices, unsigned long long normal_tex, unsigned long long tangent_tex, int64_t n,
                   const int32_t* prim, const float* bary, const float* o, const float* d, const float* tmax,
                   float* sn, float* gn, float* st, float* uv, float* p) {
    using namespace optix;
    HitGroupData hg;
    std::memset((void*)&hg, 0, sizeof(hg));
    TriangleMesh& mesh = hg.geometry_data.triangle_mesh;
    mesh.positions = (float3*)const_cast<float*>(positions);
    mesh.indices = (int3*)const_cast<int32_t*>(indices);
    mesh.normals = (float3*)const_cast<float*>(normals);
    mesh.tangents = (float3*)const_cast<float*>(tangents);
    mesh.texcoords = (float2*)const_cast<float*>(texcoords);
    Material m;
    std::memset((void*)&m, 0, sizeof(m));
    m.type = Material::ANISOGGX;
    m.normal_tex = normal_tex;
    m.tangent_tex = tangent_tex;
    m.is_tangent_space = false;
    for (int64_t i = 0; i < n; i++) {
        refshim::g_optix.sbt = &hg;
        refshim::g_optix.prim = prim[i];
        refshim::g_optix.bary = make_float2(bary[2 * i], bary[2 * i + 1]);
        refshim::g_optix.ray_o = ld3(o + 3 * i);
        refshim::g_optix.ray_d = ld3(d + 3 * i);
        refshim::g_optix.tmax = tmax[i];
        Intersection its = getHitData(m);
        st3(sn + 3 * i, its.sn);
        st3(gn + 3 * i, its.gn);
        st3(st + 3 * i, its.st);
        uv[2 * i] = its.uv.x;
        uv[2 * i + 1] = its.uv.y;
        st3(p + 3 * i, its.p);
    }
}

}  // extern "C"
