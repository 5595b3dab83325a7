// Scene construction from dl_*_desc arrays: validation, BVH build, emitter
// tables and upload.  Replaces Scene::addChild / Scene::activate /
// Mesh::activate / OCTree::build of the reference
// (src/tracer/scene/scene.cpp:19-106, src/tracer/mesh/mesh.cpp:15-45).
//
// Compiled with -ffp-contract=off: the per-face areas and the area CDF of
// every emitting mesh are computed with the reference's float operations
// (mesh.cpp:102-108, dpdf.h:70-103) so light sampling picks the same faces.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "bvh.h"
#include "internal.h"
#include "scene.h"

namespace dl {
namespace {

struct HV {
    float x, y, z;
};
inline HV hsub(HV a, HV b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline HV hcross(HV a, HV b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float hdot(HV a, HV b) {
    float s = 0;
    s += a.x * b.x;
    s += a.y * b.y;
    s += a.z * b.z;
    return s;
}
inline float hlen(HV a) { return std::sqrt(hdot(a, a)); }
inline HV hnorm(HV a) {
    float l = hlen(a);
    return {a.x / l, a.y / l, a.z / l};
}
inline HV hscale(HV a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline HV ld(const float* p) { return {p[0], p[1], p[2]}; }

// Alias table over non-negative weights: the steps of the reference's
// build_alias_map (src/tracer/emitter/envmap.cpp:111-141; one partition
// array, small entries from the front, large from the back, each small entry
// topped up from the current large one).  The normalised weights and the
// residual chain (q[k] += q[j] - 1) run in double: in the reference's float a
// long chain misstates a pick probability by up to tens of percent on maps
// with a bright sun, and the pick would no longer follow the pdf.  Returns
// the sum of the weights; with a zero sum every entry picks itself.
double alias_table(const std::vector<double>& w, std::vector<double>& q, std::vector<unsigned>& alias) {
    const unsigned size = (unsigned)w.size();
    q.assign(size, 1.0);
    alias.resize(size);
    double sum = 0.0;
    for (unsigned i = 0; i < size; ++i) sum += w[i];
    for (unsigned i = 0; i < size; ++i) alias[i] = i;
    if (!(sum > 0.0)) return 0.0;
    for (unsigned i = 0; i < size; ++i) q[i] = (double)size * w[i] / sum;
    std::vector<unsigned> part(size);
    unsigned s = 0u, large = size;
    for (unsigned i = 0; i < size; ++i) part[(q[i] < 1.0) ? (s++) : (--large)] = i;
    for (s = 0; s < large && large < size; ++s) {
        const unsigned j = part[s], k = part[large];
        alias[j] = k;
        q[k] += q[j] - 1.0;
        large = (q[k] < 1.0) ? (large + 1u) : large;
    }
    return sum;
}

float4 alias_entry(double q, unsigned alias, float prob) {
    float a;
    std::memcpy(&a, &alias, 4);
    return make_float4((float)q, a, prob, 0.f);
}

// EnvironmentMap::activate (src/tracer/emitter/envmap.cpp:59-110): the
// importance of a texel is its solid angle times max(r, g, b) (float, as the
// reference computes it; its unqualified cos of a float is the double cos);
// the alias table picks texels in proportion to it; pdf = max(r, g, b) /
// sum(importance) is the solid-angle density of a direction in the texel.
// Returns sum(importance): the integral of max(r, g, b) over the sphere.
double build_env_tables(const dl_light_desc& L, std::vector<float4>& tex, std::vector<float4>& accel) {
    const unsigned rx = (unsigned)L.env_width, ry = (unsigned)L.env_height, size = rx * ry;
    const float* px = L.env_rgb;
    const float pi = 3.14159265358979323846f;
    tex.resize(size);
    accel.resize(size);
    std::vector<double> imp(size), q;
    std::vector<unsigned> alias;
    auto maxc = [&](unsigned i) { return std::max(px[3 * i], std::max(px[3 * i + 1], px[3 * i + 2])); };
    float cos_theta0 = 1.0f;
    const float step_phi = (float)(2.0 * (double)pi) / (float)rx;
    const float step_theta = pi / (float)ry;
    for (unsigned y = 0; y < ry; ++y) {
        const float theta1 = (float)(y + 1) * step_theta;
        const float cos_theta1 = (float)std::cos((double)theta1);
        const float area = (cos_theta0 - cos_theta1) * step_phi;
        cos_theta0 = cos_theta1;
        for (unsigned x = 0; x < rx; ++x) imp[y * rx + x] = (double)(area * maxc(y * rx + x));
    }
    const double sum = alias_table(imp, q, alias);
    for (unsigned i = 0; i < size; ++i) {
        accel[i] = alias_entry(q[i], alias[i], sum > 0.0 ? (float)((double)maxc(i) / sum) : 0.0f);
        tex[i] = make_float4(px[3 * i], px[3 * i + 1], px[3 * i + 2], 0.f);
    }
    return sum;
}

void check(bool ok, const std::string& msg) {
    if (!ok) throw Error(DL_ERR_INVALID_ARG, msg);
}

}  // namespace

namespace {

// 4x4 inverse in double (Gauss-Jordan, partial pivoting), rounded to float.
bool invert4(const double* a, float* out) {
    double m[4][8];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 8; j++) m[i][j] = j < 4 ? a[4 * i + j] : (j - 4 == i ? 1.0 : 0.0);
    for (int c = 0; c < 4; c++) {
        int p = c;
        for (int r = c + 1; r < 4; r++)
            if (std::fabs(m[r][c]) > std::fabs(m[p][c])) p = r;
        if (!(std::fabs(m[p][c]) > 1e-30)) return false;
        if (p != c)
            for (int j = 0; j < 8; j++) std::swap(m[p][j], m[c][j]);
        const double inv = 1.0 / m[c][c];
        for (int j = 0; j < 8; j++) m[c][j] *= inv;
        for (int r = 0; r < 4; r++) {
            if (r == c || m[r][c] == 0.0) continue;
            const double f = m[r][c];
            for (int j = 0; j < 8; j++) m[r][j] -= f * m[c][j];
        }
    }
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) out[4 * i + j] = (float)m[i][j + 4];
    return true;
}

void matmul4(const double* a, const double* b, double* out) {
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double s = 0.0;
            for (int k = 0; k < 4; k++) s += a[4 * i + k] * b[4 * k + j];
            out[4 * i + j] = s;
        }
}

}  // namespace

void validate_camera(const dl_camera_desc& c) {
    check(c.type == DL_CAMERA_VIRTUAL || c.type == DL_CAMERA_PERSPECTIVE || c.type == DL_CAMERA_OPENCV,
          "unsupported camera type");
    check(c.width > 0 && c.height > 0 && c.width <= 65536 && c.height <= 65536, "camera resolution out of range");
    if (c.type != DL_CAMERA_VIRTUAL)
        for (int k = 0; k < 16; k++) check(std::isfinite(c.transform[k]), "camera transform must be finite");
    if (c.type != DL_CAMERA_OPENCV) check(c.fov > 0.f && c.fov < 180.f, "camera fov out of range");
    if (c.type == DL_CAMERA_PERSPECTIVE) {
        // Camera rays start at t = 1e-4 like every other render ray; the
        // reference starts them at near_clip / d.z, the same to within the
        // factor 1 / d.z only for its default near clip.
        check(std::fabs(c.near_clip - 1e-4f) <= 1e-9f, "perspective camera: only the default nearClip (1e-4) is supported");
        check(c.far_clip > c.near_clip && std::isfinite(c.far_clip), "perspective camera: farClip out of range");
    }
    if (c.type == DL_CAMERA_OPENCV)
        check(std::isfinite(c.fx) && std::isfinite(c.fy) && c.fx != 0.f && c.fy != 0.f && std::isfinite(c.cx) &&
                  std::isfinite(c.cy),
              "opencv camera: bad intrinsics");
}

// virtual.cpp:16-42; perspective.cpp:41-73 (sample-to-camera matrix, here
// composed and inverted in double); opencv.cpp:10-24 (inverse extrinsic and
// eye).
DevCamera make_camera(const dl_camera_desc& c) {
    DevCamera cam;
    std::memset(&cam, 0, sizeof(cam));
    cam.type = c.type;
    cam.w = c.width;
    cam.h = c.height;
    cam.inv_w = 1.f / c.width;
    cam.inv_h = 1.f / c.height;
    if (c.type == DL_CAMERA_PERSPECTIVE) {
        const double aspect = (double)(c.width / (float)c.height);
        const double n = c.near_clip, f = c.far_clip;
        const double recip = 1.0 / (f - n), cot = 1.0 / std::tan((double)c.fov * 0.5 * 3.14159265358979323846 / 180.0);
        const double P[16] = {cot, 0, 0, 0, 0, cot, 0, 0, 0, 0, f * recip, -n * f * recip, 0, 0, 1, 0};
        const double Sc[16] = {-0.5, 0, 0, 0, 0, -0.5 * aspect, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        const double Tr[16] = {1, 0, 0, -1, 0, 1, 0, -1.0 / aspect, 0, 0, 1, 0, 0, 0, 0, 1};
        double A[16], B[16];
        matmul4(Sc, Tr, A);
        matmul4(A, P, B);
        if (!invert4(B, cam.S)) throw Error(DL_ERR_INVALID_ARG, "perspective camera: singular projection");
        for (int k = 0; k < 16; k++) cam.T[k] = c.transform[k];
        cam.far_clip = c.far_clip;
        return cam;
    }
    if (c.type == DL_CAMERA_OPENCV) {
        double E[16];
        for (int k = 0; k < 16; k++) E[k] = c.transform[k];
        if (!invert4(E, cam.T)) throw Error(DL_ERR_INVALID_ARG, "opencv camera: singular extrinsic");
        // eye = inverse extrinsic * (0, 0, 0, 1)
        for (int i = 0; i < 3; i++) cam.eye[i] = cam.T[4 * i + 3];
        cam.fx = c.fx;
        cam.fy = c.fy;
        cam.cx = c.cx;
        cam.cy = c.cy;
        return cam;
    }
    const float pi = 3.14159265358979323846f;
    float aspect = c.width / (float)c.height;
    HV eye = ld(c.eye), look = ld(c.lookat), up = ld(c.up);
    HV W = hsub(look, eye);
    float wlen = hlen(W);
    HV U = hnorm(hcross(W, up));
    HV V = hnorm(hcross(U, W));
    float vlen = wlen * tanf(0.5f * c.fov * pi / 180.f);
    V = hscale(V, vlen);
    U = hscale(U, vlen * aspect);
    cam.eye[0] = eye.x; cam.eye[1] = eye.y; cam.eye[2] = eye.z;
    cam.U[0] = U.x; cam.U[1] = U.y; cam.U[2] = U.z;
    cam.V[0] = V.x; cam.V[1] = V.y; cam.V[2] = V.z;
    cam.W[0] = W.x; cam.W[1] = W.y; cam.W[2] = W.z;
    return cam;
}

void validate_scene(const dl_mesh_desc* meshes, int32_t nm, const dl_material_desc* mats, int32_t nmat,
                    const dl_light_desc* lights, int32_t nl, const dl_camera_desc* cam) {
    check(nm >= 0 && nmat >= 0 && nl >= 0, "negative count");
    check(nm == 0 || meshes, "meshes is NULL");
    check(nmat == 0 || mats, "materials is NULL");
    check(nl == 0 || lights, "lights is NULL");
    check(cam != nullptr, "camera is NULL");
    validate_camera(*cam);
    int64_t total = 0;
    for (int i = 0; i < nm; i++) {
        const dl_mesh_desc& m = meshes[i];
        check(m.num_vertices >= 0 && m.num_triangles >= 0, "mesh " + std::to_string(i) + ": negative size");
        check(m.num_triangles == 0 || (m.positions && m.indices), "mesh " + std::to_string(i) + ": NULL arrays");
        check(m.material >= 0 && m.material < nmat, "mesh " + std::to_string(i) + ": material out of range");
        check(m.light >= -1 && m.light < nl, "mesh " + std::to_string(i) + ": light out of range");
        if (m.light >= 0)
            check(lights[m.light].type == DL_LIGHT_AREA && lights[m.light].mesh == i,
                  "mesh " + std::to_string(i) + ": light is not an area light of this mesh");
        for (int64_t k = 0; k < 3 * m.num_triangles; k++)
            check(m.indices[k] < (uint64_t)m.num_vertices, "mesh " + std::to_string(i) + ": vertex index out of range");
        for (int64_t k = 0; k < 3 * m.num_vertices; k++)
            check(std::isfinite(m.positions[k]), "mesh " + std::to_string(i) + ": non-finite vertex");
        total += m.num_triangles;
    }
    check(total < (int64_t)1 << 27, "too many triangles (limit 2^27)");
    for (int i = 0; i < nmat; i++) {
        const dl_material_desc& m = mats[i];
        check(m.type >= DL_MAT_DIFFUSE && m.type <= DL_MAT_ANISO_GGX, "material " + std::to_string(i) + ": bad type");
        if (m.type == DL_MAT_MICROFACET) check(m.alpha[0] > 0.f, "microfacet alpha must be > 0");
        if (m.type == DL_MAT_ANISO_GGX) check(m.alpha[0] > 0.f && m.alpha[1] > 0.f, "aniso_ggx alpha must be > 0");
        const std::string who = "material " + std::to_string(i) + ": ";
        const dl_texture_desc* slots[5] = {&m.albedo_texture, &m.specular_texture, &m.alpha_texture,
                                           &m.normal_texture, &m.tangent_texture};
        for (int k = 0; k < 5; k++) {
            const dl_texture_desc& t = *slots[k];
            if (!t.rgb) continue;
            // which textures each BSDF reads (diffuse.cu:15-20, aniso_ggx.cu:19-35)
            check(m.type == DL_MAT_ANISO_GGX || (m.type == DL_MAT_DIFFUSE && k == 0),
                  who + "this BSDF takes no such texture");
            check(t.width > 0 && t.height > 0 && (int64_t)t.width * t.height <= ((int64_t)1 << 26),
                  who + "texture size out of range");
            for (int64_t q = 0; q < 3 * (int64_t)t.width * t.height; q++)
                check(std::isfinite(t.rgb[q]), who + "texture values must be finite");
        }
    }
    int num_env = 0;
    for (int l = 0; l < nl; l++) {
        const dl_light_desc& L = lights[l];
        if (L.type == DL_LIGHT_AREA) {
            check(L.mesh >= 0 && L.mesh < nm, "light " + std::to_string(l) + ": mesh out of range");
            check(meshes[L.mesh].light == l, "light " + std::to_string(l) + ": mesh does not point back to it");
            check(meshes[L.mesh].num_triangles > 0, "light " + std::to_string(l) + ": emitting mesh is empty");
        } else if (L.type == DL_LIGHT_POINT) {
        } else if (L.type == DL_LIGHT_ENVMAP) {
            std::string who = "light " + std::to_string(l) + ": ";
            check(++num_env == 1, who + "more than one envmap in the scene");
            check(L.env_rgb != nullptr, who + "env_rgb is NULL");
            check(L.env_width > 0 && L.env_height > 0 && (int64_t)L.env_width * L.env_height <= ((int64_t)1 << 26),
                  who + "envmap size out of range");
            check(std::isfinite(L.env_scale), who + "envmap scale is not finite");
            for (int64_t k = 0; k < 3 * (int64_t)L.env_width * L.env_height; k++)
                check(std::isfinite(L.env_rgb[k]) && L.env_rgb[k] >= 0.f,
                      who + "envmap texels must be finite and non-negative");
        } else {
            throw Error(DL_ERR_INVALID_ARG, "light " + std::to_string(l) + ": bad type");
        }
    }
}

void build_scene(dl_scene* S, const dl_mesh_desc* meshes, int32_t nm, const dl_material_desc* mats, int32_t nmat,
                 const dl_light_desc* lights, int32_t nl, const dl_camera_desc* cam) {
    validate_scene(meshes, nm, mats, nmat, lights, nl, cam);
    cudaStream_t st = S->ctx->stream;
    int64_t ntri = 0, nvert = 0;
    for (int i = 0; i < nm; i++) {
        ntri += meshes[i].num_triangles;
        nvert += meshes[i].num_vertices;
    }
    std::vector<float> tri9((size_t)ntri * 9);
    std::vector<int4> vidx_orig((size_t)ntri);
    std::vector<float4> normals((size_t)std::max<int64_t>(nvert, 1));
    std::vector<float2> texcoords((size_t)std::max<int64_t>(nvert, 1));
    std::vector<DevMesh> dmesh(std::max(nm, 1));
    int64_t t = 0, vo = 0;
    for (int i = 0; i < nm; i++) {
        const dl_mesh_desc& m = meshes[i];
        for (int64_t f = 0; f < m.num_triangles; f++, t++) {
            for (int k = 0; k < 3; k++) {
                uint32_t vi = m.indices[3 * f + k];
                std::memcpy(&tri9[9 * t + 3 * k], m.positions + 3 * vi, 12);
            }
            vidx_orig[t] = make_int4((int)(vo + m.indices[3 * f]), (int)(vo + m.indices[3 * f + 1]),
                                     (int)(vo + m.indices[3 * f + 2]), i);
        }
        for (int64_t v = 0; v < m.num_vertices; v++) {
            if (m.normals)
                normals[vo + v] = make_float4(m.normals[3 * v], m.normals[3 * v + 1], m.normals[3 * v + 2], 0.f);
            else
                normals[vo + v] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        dmesh[i].material = m.material;
        dmesh[i].light = m.light;
        dmesh[i].has_normals = m.normals != nullptr;
        dmesh[i].has_texcoords = m.texcoords != nullptr;
        for (int64_t v = 0; v < m.num_vertices; v++)
            texcoords[vo + v] = m.texcoords ? make_float2(m.texcoords[2 * v], m.texcoords[2 * v + 1])
                                            : make_float2(0.f, 0.f);
        vo += m.num_vertices;
    }
    BvhBuildOptions bo;
    BvhResult bvh = build_bvh(tri9.data(), ntri, bo);
    // the traversal kernels push at most one entry per inner level
    if (bvh.depth - 1 > kStackSize)
        throw Error(DL_ERR_INVALID_ARG, "BVH depth " + std::to_string(bvh.depth) + " exceeds the traversal stack (" +
                                            std::to_string(kStackSize) + " entries)");
    std::vector<int4> vidx((size_t)std::max<int64_t>(ntri, 1));
    for (size_t k = 0; k < bvh.tri_order.size(); k++) vidx[k] = vidx_orig[bvh.tri_order[k]];

    std::vector<DevMaterial> dmat(std::max(nmat, 1));
    std::vector<float4> texels;
    std::vector<int64_t> tex_offset;
    std::vector<DevTexture> dtex;
    for (int i = 0; i < nmat; i++) {
        const dl_material_desc& m = mats[i];
        DevMaterial& d = dmat[i];
        d.type = m.type;
        for (int k = 0; k < 3; k++) {
            d.albedo[k] = m.albedo[k];
            d.specular[k] = m.specular[k];
        }
        d.ax = m.alpha[0];
        d.ay = m.alpha[1];
        d.int_ior = m.int_ior;
        d.ext_ior = m.ext_ior;
        d.ks = 1 - std::max(std::max(m.albedo[0], m.albedo[1]), m.albedo[2]);
        const dl_texture_desc* slots[kTexSlots] = {&m.albedo_texture, &m.specular_texture, &m.alpha_texture,
                                                   &m.normal_texture, &m.tangent_texture};
        d.has_tex = 0;
        for (int k = 0; k < kTexSlots; k++) {
            d.tex[k] = -1;
            const dl_texture_desc& t = *slots[k];
            if (!t.rgb) continue;
            DevTexture dt;
            dt.texels = nullptr;  // set after the upload
            dt.w = t.width;
            dt.h = t.height;
            tex_offset.push_back((int64_t)texels.size());
            for (int64_t q = 0; q < (int64_t)t.width * t.height; q++)
                texels.push_back(make_float4(t.rgb[3 * q], t.rgb[3 * q + 1], t.rgb[3 * q + 2], 0.f));
            d.tex[k] = (int)dtex.size();
            dtex.push_back(dt);
            d.has_tex = 1;
        }
    }

    std::vector<DevLight> dlights(std::max(nl, 1));
    std::vector<float4> etris;
    std::vector<float> ecdf;
    for (int l = 0; l < nl; l++) {
        const dl_light_desc& L = lights[l];
        DevLight& d = dlights[l];
        std::memset(&d, 0, sizeof(d));
        d.type = L.type;
        d.mesh = L.mesh;
        for (int k = 0; k < 3; k++) {
            d.radiance[k] = L.radiance[k];
            d.position[k] = L.position[k];
        }
        if (L.type == DL_LIGHT_AREA) {
            const dl_mesh_desc& m = meshes[L.mesh];
            d.tri_begin = (int)(etris.size() / 6);
            d.tri_count = (int)m.num_triangles;
            d.cdf_begin = (int)ecdf.size();
            d.has_normals = m.normals != nullptr;
            // DiscretePDF over face areas (mesh.cpp:21-28, dpdf.h:70-103)
            std::vector<float> cdf;
            cdf.push_back(0.0f);
            for (int64_t f = 0; f < m.num_triangles; f++) {
                HV p[3], n[3];
                for (int k = 0; k < 3; k++) {
                    uint32_t vi = m.indices[3 * f + k];
                    p[k] = ld(m.positions + 3 * vi);
                    n[k] = m.normals ? ld(m.normals + 3 * vi) : HV{0, 0, 0};
                }
                float area = 0.5f * hlen(hcross(hsub(p[1], p[0]), hsub(p[2], p[0])));
                cdf.push_back(cdf.back() + area);
                for (int k = 0; k < 3; k++) etris.push_back(make_float4(p[k].x, p[k].y, p[k].z, 0.f));
                for (int k = 0; k < 3; k++) etris.push_back(make_float4(n[k].x, n[k].y, n[k].z, 0.f));
            }
            float sum = cdf.back();
            float norm = 0.0f;
            if (sum > 0) {
                norm = 1.0f / sum;
                for (size_t i = 1; i < cdf.size(); ++i) cdf[i] *= norm;
                cdf.back() = 1.0f;
            }
            d.pA = norm;
            ecdf.insert(ecdf.end(), cdf.begin(), cdf.end());
        }
    }
    int env_light = -1;
    double env_integral = 0.0;
    std::vector<float4> env_tex, env_accel;
    for (int l = 0; l < nl; l++) {
        if (lights[l].type != DL_LIGHT_ENVMAP) continue;
        env_light = l;
        env_integral = build_env_tables(lights[l], env_tex, env_accel);
    }
    if (env_tex.empty()) {
        env_tex.push_back(make_float4(0.f, 0.f, 0.f, 0.f));
        env_accel.push_back(make_float4(1.f, 0.f, 0.f, 0.f));
    }
    S->env_tex.upload(env_tex, st);
    S->env_accel.upload(env_accel, st);
    // power-proportional emitter pick (DL_RENDER_POWER_LIGHT_PICK)
    std::vector<double> power(std::max(nl, 1), 0.0), pq;
    std::vector<unsigned> palias;
    {
        const double kPi = 3.14159265358979323846;
        // bounding box of every vertex of every mesh; R = half its diagonal
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        bool any = false;
        for (int i = 0; i < nm; i++)
            for (int64_t k = 0; k < 3 * meshes[i].num_vertices; k++) {
                lo[k % 3] = std::min(lo[k % 3], (double)meshes[i].positions[k]);
                hi[k % 3] = std::max(hi[k % 3], (double)meshes[i].positions[k]);
                any = true;
            }
        double r2 = 0.0;
        if (any)
            for (int k = 0; k < 3; k++) r2 += 0.25 * (hi[k] - lo[k]) * (hi[k] - lo[k]);
        for (int k = 0; k < 3; k++) {
            double ext = any ? hi[k] - lo[k] : 0.0;
            S->dev.bb_lo[k] = any ? (float)lo[k] : 0.f;
            S->dev.bb_inv_ext[k] = ext > 0.0 ? (float)(1.0 / ext) : 0.f;
        }
        for (int l = 0; l < nl; l++) {
            const dl_light_desc& L = lights[l];
            double m = std::max(L.radiance[0], std::max(L.radiance[1], L.radiance[2]));
            if (L.type == DL_LIGHT_AREA) {
                double area = 0.0;
                const dl_mesh_desc& me = meshes[L.mesh];
                for (int64_t f = 0; f < me.num_triangles; f++) {
                    HV p[3];
                    for (int k = 0; k < 3; k++) p[k] = ld(me.positions + 3 * me.indices[3 * f + k]);
                    area += (double)(0.5f * hlen(hcross(hsub(p[1], p[0]), hsub(p[2], p[0]))));
                }
                power[l] = kPi * area * std::max(m, 0.0);
            } else if (L.type == DL_LIGHT_POINT) {
                power[l] = 4.0 * kPi * std::max(m, 0.0);
            } else if (L.type == DL_LIGHT_ENVMAP) {
                power[l] = kPi * r2 * env_integral * (double)std::fabs(L.env_scale);
            }
        }
        power.resize(std::max(nl, 1));
        if (nl == 0) power[0] = 1.0;
    }
    std::vector<float4> pick(power.size());
    {
        double psum = alias_table(power, pq, palias);
        for (size_t l = 0; l < power.size(); l++)
            pick[l] = alias_entry(pq[l], palias[l],
                                  psum > 0.0 ? (float)(power[l] / psum) : 1.0f / (float)power.size());
    }
    S->light_pick.upload(pick, st);

    // the closest-hit kernel routes a hit to its material's queue from the
    // triangle record it has just tested (second vertex's w)
    for (size_t k = 0; k < bvh.tris.size(); k++)
        bvh.tris[k].mat_type = dmat[dmesh[vidx[k].w].material].type;
    S->nodes.upload(bvh.nodes, st);
    S->tris.upload(bvh.tris, st);
    S->tri_vidx.upload(vidx, st);
    S->normals.upload(normals, st);
    S->texcoords.upload(texcoords, st);
    if (texels.empty()) texels.push_back(make_float4(0.f, 0.f, 0.f, 0.f));
    S->texels.upload(texels, st);
    for (size_t k = 0; k < dtex.size(); k++) dtex[k].texels = S->texels.as<float4>() + tex_offset[k];
    if (dtex.empty()) dtex.push_back(DevTexture{nullptr, 0, 0});
    S->textures.upload(dtex, st);
    S->meshes.upload(dmesh, st);
    S->materials.upload(dmat, st);
    S->lights.upload(dlights, st);
    if (etris.empty()) etris.push_back(make_float4(0.f, 0.f, 0.f, 0.f));
    if (ecdf.empty()) ecdf.push_back(0.f);
    S->emit_tris.upload(etris, st);
    S->emit_cdf.upload(ecdf, st);
    DL_CUDA(cudaStreamSynchronize(st));

    DevScene& D = S->dev;
    D.nodes = S->nodes.as<float4>();
    D.tris = S->tris.as<float4>();
    D.tri_vidx = S->tri_vidx.as<int4>();
    D.normals = S->normals.as<float4>();
    D.meshes = S->meshes.as<DevMesh>();
    D.materials = S->materials.as<DevMaterial>();
    D.lights = S->lights.as<DevLight>();
    D.emit_tris = S->emit_tris.as<float4>();
    D.emit_cdf = S->emit_cdf.as<float>();
    D.textures = S->textures.as<DevTexture>();
    D.texcoords = S->texcoords.as<float2>();
    D.num_tris = (int)ntri;
    D.num_nodes = (int)bvh.nodes.size();
    D.num_lights = nl;
    D.cam = make_camera(*cam);
    D.light_pick = S->light_pick.as<float4>();
    D.env_tex = S->env_tex.as<float4>();
    D.env_accel = S->env_accel.as<float4>();
    D.env_light = env_light;
    D.env_w = env_light >= 0 ? lights[env_light].env_width : 1;
    D.env_h = env_light >= 0 ? lights[env_light].env_height : 1;
    D.env_visual = env_light >= 0 ? (lights[env_light].env_visual != 0) : 0;
    D.env_scale = env_light >= 0 ? lights[env_light].env_scale : 0.f;
    for (int k = 0; k < 3; k++) D.env_bg[k] = env_light >= 0 ? lights[env_light].env_background[k] : 0.f;
    S->tri_order = bvh.tri_order;

    dl_scene_info& I = S->info;
    I.num_triangles = ntri;
    I.num_bvh_nodes = (int64_t)bvh.nodes.size();
    I.num_meshes = nm;
    I.num_materials = nmat;
    I.num_lights = nl;
    I.width = cam->width;
    I.height = cam->height;
    I.bvh_depth = bvh.depth;
    I.bvh_build_seconds = bvh.seconds;
    I.bvh_sah_cost = bvh.sah_cost;
    I.device_bytes = (int64_t)(S->nodes.bytes + S->tris.bytes + S->tri_vidx.bytes + S->normals.bytes +
                               S->meshes.bytes + S->materials.bytes + S->lights.bytes + S->emit_tris.bytes +
                               S->emit_cdf.bytes + S->env_tex.bytes + S->env_accel.bytes +
                               S->light_pick.bytes);
    dl_render_opts& O = S->defaults;
    std::memset(&O, 0, sizeof(O));
    O.spp = 1;
    O.max_depth = 0;
    O.rr_depth = 3;
    O.filter = DL_FILTER_GAUSSIAN;
}

}  // namespace dl
