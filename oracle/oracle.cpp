// CPU restatement of the xuxmin/DrawLab path-tracer hot path.
//
// TEST INFRASTRUCTURE ONLY (see oracle.h): the oracle the GPU path is tested
// against, and the timed CPU baseline.  Nothing in the product links this file.
//
// It restates, step for step and in the same float/double operation order,
// the reference CPU backend (paths relative to the reference project root):
//   octree build / closest hit / any hit  src/tracer/accel/octree.cpp:7-212
//   slab test                             include/core/math/bbox.h:258-315
//   Moller-Trumbore, area sampling        src/tracer/mesh/mesh.cpp:102-246
//   path integrator (NEE + MIS + RR)      src/tracer/integrator/path.cpp:13-108
//   emitter pick, shadow test, pdf        src/tracer/scene/scene.cpp:139-179
//   area / point emitters                 src/tracer/emitter/{area,point}.cpp
//   diffuse, mirror, dielectric, Beckmann src/tracer/bsdf/*.cpp
//   warps, fresnel, refract, reflect      src/core/math/{wrap,math}.cpp
//   shading frame                         include/core/math/frame.h:28-48
//   discrete pdf                          include/core/math/dpdf.h:95-136
//   virtual camera                        src/tracer/camera/virtual.cpp:16-65
//   film splat, merge, normalise          src/core/bitmap/block.cpp:10-177
//   Gaussian / box filters                src/tracer/rfilter/rfilter.cpp
//   pcg32 sampler, block loop             src/tracer/sampler/independent.cpp,
//                                         src/tracer/backend/cpu_renderer.cpp
// and, in the same style, the parts the reference has only in OptiX CUDA:
//   GGX / anisotropic GGX                 src/optix/cuda/material/aniso_ggx.cu,
//                                         include/optix/math/wrap.h:54-77,
//                                         include/optix/math/onb.h:11-43
//   point light with cosine (fix flag)    include/optix/light/point.h:15-42
//   envmap emitter and miss shading       include/optix/light/envmap.h:25-94,
//                                         src/tracer/emitter/envmap.cpp:59-141,
//                                         src/optix/cuda/miss.cu:11-49
// and the renderer's own option of a power-proportional emitter pick.
//
// Where the reference calls an unqualified libm function (cos, sin, atan,
// log, exp, acos) on a float, C++ overload resolution picks the double
// version; this file calls the double version there too, so that the
// restatement reproduces the reference's results bit for bit.
//
// Compiled with -ffp-contract=off (no fused multiply-add).
#include "oracle.h"

#include <stdexcept>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>
#include <thread>
#include <utility>
#include <vector>

namespace {

const float kEps = 0.0001f;                   // M_EPSILON (include/core/math/math.h:14)
const float kPi = 3.14159265358979323846f;    // M_PI redefined as float (math.h:17)
const float kInvPi = 0.31830988618379067154f;
const float kInvTwoPi = 0.15915494309189533577f;
const float kInf = std::numeric_limits<float>::infinity();

// ------------------------------------------------------------ vector math
struct V3 {
    float x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator-(V3 a) { return V3(-a.x, -a.y, -a.z); }
inline V3 operator*(V3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(float s, V3 a) { return V3(s * a.x, s * a.y, s * a.z); }
inline V3 operator/(V3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
inline V3 mul(V3 a, V3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float dot(V3 a, V3 b) {
    float s = 0;
    s += a.x * b.x;
    s += a.y * b.y;
    s += a.z * b.z;
    return s;
}
inline V3 cross(V3 a, V3 b) {
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalized(V3 a) {
    float l = length(a);
    return V3(a.x / l, a.y / l, a.z / l);
}
inline float maxc(V3 a) { return std::max(std::max(a.x, a.y), a.z); }
inline V3 vmin(V3 a, V3 b) { return V3(std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)); }
inline V3 vmax(V3 a, V3 b) { return V3(std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)); }
inline V3 ld3(const float* p) { return V3(p[0], p[1], p[2]); }

struct P2 {
    float x, y;
};

// ----------------------------------------------------------------- pcg32
// PCG32 (O'Neill 2014, XSH-RR) with the wjakob/pcg32 seeding and float
// construction used by the reference sampler (independent.cpp:31-45).
struct Pcg32 {
    uint64_t state = 0x853c49e6748fea9bULL, inc = 0xda3e39cb94b95bdbULL;
    void seed(uint64_t initstate, uint64_t initseq) {
        state = 0u;
        inc = (initseq << 1u) | 1u;
        next_u32();
        state += initstate;
        next_u32();
    }
    uint32_t next_u32() {
        uint64_t old = state;
        state = old * 0x5851f42d4c957f2dULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((~rot + 1u) & 31));
    }
    float next_float() {
        union { uint32_t u; float f; } c;
        c.u = (next_u32() >> 9) | 0x3f800000u;
        return c.f - 1.0f;
    }
    // Independent::next2D constructs Point2f(nextFloat(), nextFloat()); the
    // compiled reference (g++, x86-64) evaluates the two arguments right to
    // left, so the first draw lands in y.
    P2 next2d() {
        float first = next_float();
        float second = next_float();
        return P2{second, first};
    }
    float next1d() { return next_float(); }
};

inline uint64_t splitmix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// ------------------------------------------------------------------ ray/box
struct Ray {
    V3 o, d, drcp;
    float mint, maxt;
};
inline Ray make_ray(V3 o, V3 d, float mint = kEps, float maxt = kInf) {
    Ray r;
    r.o = o;
    r.d = d;
    r.drcp = V3(1 / d.x, 1 / d.y, 1 / d.z);
    r.mint = mint;
    r.maxt = maxt;
    return r;
}

struct BBox {
    V3 mn{kInf, kInf, kInf}, mx{-kInf, -kInf, -kInf};
    void expand(V3 p) { mn = vmin(mn, p); mx = vmax(mx, p); }
    void expand(const BBox& b) { mn = vmin(mn, b.mn); mx = vmax(mx, b.mx); }
    V3 center() const { return (mx + mn) * 0.5f; }
    V3 corner(int i) const {
        return V3((i & 1) ? mx.x : mn.x, (i & 2) ? mx.y : mn.y, (i & 4) ? mx.z : mn.z);
    }
    bool overlaps(const BBox& b) const {
        return b.mn.x <= mx.x && b.mn.y <= mx.y && b.mn.z <= mx.z && b.mx.x >= mn.x &&
               b.mx.y >= mn.y && b.mx.z >= mn.z;
    }
    // bbox.h:288-315 (nearT/farT left as computed when it returns false)
    bool slab(const Ray& r, float& nearT, float& farT) const {
        nearT = -kInf;
        farT = kInf;
        for (int i = 0; i < 3; i++) {
            float o = r.o[i], lo = mn[i], hi = mx[i];
            if (r.d[i] == 0) {
                if (o < lo || o > hi) return false;
            } else {
                float t1 = (lo - o) * r.drcp[i];
                float t2 = (hi - o) * r.drcp[i];
                if (t1 > t2) std::swap(t1, t2);
                nearT = std::max(t1, nearT);
                farT = std::min(t2, farT);
                if (!(nearT <= farT)) return false;
            }
        }
        return true;
    }
    // bbox.h:258-285
    bool hit(const Ray& r) const {
        float n, f;
        if (!slab(r, n, f)) return false;
        return r.mint <= f && n <= r.maxt;
    }
};

// -------------------------------------------------------------- discrete pdf
struct DPdf {
    std::vector<float> cdf{0.0f};
    float sum = 0, norm = 0;
    void append(float v) { cdf.push_back(cdf.back() + v); }
    void normalize() {
        sum = cdf.back();
        if (sum > 0) {
            norm = 1.0f / sum;
            for (size_t i = 1; i < cdf.size(); ++i) cdf[i] *= norm;
            cdf.back() = 1.0f;
        } else {
            norm = 0.0f;
        }
    }
    size_t sample(float x) const {
        auto it = std::lower_bound(cdf.begin(), cdf.end(), x);
        size_t idx = (size_t)std::max((ptrdiff_t)0, (ptrdiff_t)(it - cdf.begin()) - 1);
        return std::min(idx, cdf.size() - 2);
    }
    size_t sample_reuse(float& x) const {
        size_t idx = sample(x);
        x = (x - cdf[idx]) / (cdf[idx + 1] - cdf[idx]);
        return idx;
    }
};

// ---------------------------------------------------------------- frames
struct Frame {
    V3 t, b, n;
};
// frame.h:113-123
inline Frame make_frame(V3 n) {
    Frame f;
    f.n = n;
    V3 t;
    if (std::abs((double)n.z - 1.0) > kEps && std::abs((double)n.z + 1.0) > kEps)
        t = V3(0.0f, 0.0f, 1.0f);
    else
        t = V3(1.0f, 0.0f, 0.0f);
    V3 b = normalized(cross(n, t));
    f.b = b;
    f.t = cross(b, n);
    return f;
}
// Onb(normal, tangent = 0) of include/optix/math/onb.h:11-33 (frame used by
// the aniso_ggx material, whose only working form is the OptiX one).
inline Frame make_onb(V3 n) {
    Frame f;
    f.n = n;
    V3 bn;
    if (std::fabs(n.x) > std::fabs(n.z))
        bn = V3(-n.y, n.x, 0.0f);
    else
        bn = V3(0.0f, -n.z, n.y);
    f.b = normalized(bn);
    f.t = cross(f.b, n);
    return f;
}
// Onb(normal, tangent) with a non-zero tangent (onb.h:29-32)
inline Frame make_onb_t(V3 n, V3 t) {
    if (t.x == 0.f && t.y == 0.f && t.z == 0.f) return make_onb(n);
    Frame f;
    f.n = n;
    f.t = t;
    f.b = normalized(cross(n, t));
    return f;
}
inline V3 to_local(const Frame& f, V3 v) { return V3(dot(v, f.t), dot(v, f.b), dot(f.n, v)); }
inline V3 to_world(const Frame& f, V3 v) { return f.t * v.x + f.b * v.y + f.n * v.z; }
inline float tan_theta(V3 v) {
    float temp = 1 - v.z * v.z;
    if (temp <= 0.0f) return 0.0f;
    return std::sqrt(temp) / v.z;
}

// ----------------------------------------------------------------- warps
// src/core/math/wrap.cpp (unqualified libm calls resolve to double)
inline P2 square_to_uniform_disk(P2 s) {
    float r = (float)::sqrt((double)s.x);
    float theta = 2 * kPi * s.y;
    return P2{(float)(r * ::cos((double)theta)), (float)(r * ::sin((double)theta))};
}
inline V3 square_to_cosine_hemisphere(P2 s) {
    P2 p = square_to_uniform_disk(s);
    float sum = p.x * p.x + p.y * p.y;
    float z = (float)::sqrt((double)(1 - sum));
    return V3(p.x, p.y, z);
}
inline float cosine_hemisphere_pdf(V3 v) { return v.z <= 0 ? 0 : v.z * kInvPi; }
inline V3 square_to_beckmann(P2 s, float alpha) {
    float theta = (float)::atan(::sqrt(-alpha * alpha * ::log((double)(1 - s.x))));
    float phi = 2 * kPi * s.y;
    double st = ::sin((double)theta);
    return V3((float)(st * ::cos((double)phi)), (float)(st * ::sin((double)phi)),
              (float)::cos((double)theta));
}
inline float beckmann_pdf(V3 m, float alpha) {
    if (m.z <= 0) return 0;
    float c = m.z;
    float tan2 = (1 - c * c) / (c * c);
    double p = kInvTwoPi * (2 * ::exp((double)(-tan2 / (alpha * alpha)))) /
               (double)(alpha * alpha * c * c * c);
    return (float)p;
}
inline V3 square_to_uniform_triangle(P2 s) {
    float t = (float)::sqrt((double)(1.f - s.x));
    return V3(1 - t, t * s.y, t - t * s.y);
}

// src/core/math/math.cpp:8-51
float fresnel(float cosI, float extIOR, float intIOR) {
    float etaI = extIOR, etaT = intIOR;
    if (extIOR == intIOR) return 0.0f;
    if (cosI < 0.0f) {
        std::swap(etaI, etaT);
        cosI = -cosI;
    }
    float eta = etaI / etaT, sinT2 = eta * eta * (1 - cosI * cosI);
    if (sinT2 > 1.0f) return 1.0f;
    float cosT = std::sqrt(1.0f - sinT2);
    float Rs = (etaI * cosI - etaT * cosT) / (etaI * cosI + etaT * cosT);
    float Rp = (etaT * cosI - etaI * cosT) / (etaT * cosI + etaI * cosT);
    return (Rs * Rs + Rp * Rp) / 2.0f;
}
V3 refract(V3 wi, float eta) {
    float cosI = wi.z;
    bool outside = cosI > 0.f;
    eta = outside ? eta : 1 / eta;
    float cosT2 = 1 - eta * eta * (1 - cosI * cosI);
    float cosT = (float)::sqrt((double)cosT2);
    cosT = outside ? -cosT : cosT;
    return V3(-eta * wi.x, -eta * wi.y, cosT);
}
inline V3 reflect(V3 wi, V3 n) { return (2 * dot(wi, n)) * n - wi; }

// ------------------------------------------------------------------ scene
enum Measure { kUnknown = 0, kSolidAngle = 1, kDiscrete = 2 };

struct Material {
    int type;
    V3 albedo, specular;
    float ax, ay;
    float int_ior, ext_ior;
    float ks;  // microfacet: 1 - max(kd)
    int tex[5] = {-1, -1, -1, -1, -1};  // albedo, specular, alpha, normal, tangent texture; -1 = none
    bool has_tex = false;
};

struct Texture {
    int w = 0, h = 0;
    std::vector<float> rgb;  // row k at t = (k + 0.5) / h
};

struct Mesh {
    std::vector<float> V, N, UV;
    std::vector<uint32_t> F;
    int material = 0, light = -1;
    int64_t prim_offset = 0;
    DPdf dpdf;
    uint32_t tri_count() const { return (uint32_t)(F.size() / 3); }
    V3 pos(size_t f, int k) const {
        uint32_t p = F[3 * f + k];
        return V3(V[3 * p], V[3 * p + 1], V[3 * p + 2]);
    }
    V3 nrm(size_t f, int k) const {
        if (N.empty()) return V3(0, 0, 0);
        uint32_t p = F[3 * f + k];
        return V3(N[3 * p], N[3 * p + 1], N[3 * p + 2]);
    }
    BBox tri_bbox(size_t f) const {
        BBox b;
        b.mn = b.mx = pos(f, 0);
        b.expand(pos(f, 1));
        b.expand(pos(f, 2));
        return b;
    }
    float area(size_t f) const {
        V3 p0 = pos(f, 0), p1 = pos(f, 1), p2 = pos(f, 2);
        return 0.5f * length(cross(p1 - p0, p2 - p0));
    }
    // mesh.cpp:180-220
    bool intersect(size_t f, const Ray& ray, float& u, float& v, float& t) const {
        V3 p0 = pos(f, 0), p1 = pos(f, 1), p2 = pos(f, 2);
        V3 e1 = p1 - p0, e2 = p2 - p0;
        V3 pvec = cross(ray.d, e2);
        float det = dot(e1, pvec);
        if (det > -1e-8f && det < 1e-8f) return false;
        float inv = 1.0f / det;
        V3 tvec = ray.o - p0;
        u = dot(tvec, pvec) * inv;
        if (u < 0.0 || u > 1.0) return false;
        V3 qvec = cross(tvec, e1);
        v = dot(ray.d, qvec) * inv;
        if (v < 0.0 || u + v > 1.0) return false;
        t = dot(e2, qvec) * inv;
        return t >= ray.mint && t <= ray.maxt;
    }
    // mesh.cpp:222-244
    void sample_position(P2 s, V3& p, V3& n) const {
        size_t f = dpdf.sample_reuse(s.x);
        V3 p0 = pos(f, 0), p1 = pos(f, 1), p2 = pos(f, 2);
        V3 b = square_to_uniform_triangle(s);
        p = b.x * p0 + b.y * p1 + b.z * p2;
        if (!N.empty())
            n = b.x * nrm(f, 0) + b.y * nrm(f, 1) + b.z * nrm(f, 2);
        else
            n = cross(p1 - p0, p2 - p1);
        n = normalized(n);
    }
};

struct Light {
    int type;
    int mesh;
    V3 radiance, position;
    // envmap (include/optix/light/envmap.h, src/tracer/emitter/envmap.cpp)
    int env_w = 0, env_h = 0;
    float env_scale = 1.f;
    bool env_visual = true;
    V3 env_bg;
    std::vector<float> env_rgb;      // rows from the +y pole down
    std::vector<float> env_q, env_pdf;
    std::vector<uint32_t> env_alias;
    double env_sum = 0.0;            // integral of max(r, g, b) over the sphere
};

struct Node {
    BBox box;
    int child[8];
    std::vector<std::pair<int, int>> tris;  // non-empty: leaf
};

struct Hit {
    V3 p;
    float t = 0;
    P2 uv{0, 0};
    Frame sh, geo;
    int mesh = -1;
    int64_t prim = -1;
    P2 tuv{0, 0};  // texture coordinates ((0, 0) without mesh texcoords)
    V3 tan;        // aniso_ggx: shading tangent from a tangent map (0: none)
};

struct Camera {
    int w, h;
    V3 eye, U, V, W;
    float inv_w, inv_h;
    int type = DL_CAMERA_VIRTUAL;
    float S[16], T[16];  // perspective: sample-to-camera, camera-to-world; opencv: T = inverse extrinsic
    float far_clip = 0.f;
    float fx = 0.f, fy = 0.f, cx = 0.f, cy = 0.f;
};

struct Filter {
    float radius;
    int border;
    float table[33];
    float lookup;
};

struct Scene {
    std::vector<Mesh> meshes;
    std::vector<Material> mats;
    std::vector<Texture> textures;
    std::vector<Light> lights;
    int env_light = -1;
    // power-proportional emitter pick (DL_RENDER_POWER_LIGHT_PICK)
    std::vector<float> pick_q, pick_prob;
    std::vector<uint32_t> pick_alias;
    std::vector<Node> nodes;
    int root = -1;
    Camera cam;
    Filter filter;
};

thread_local std::string g_error;

// ---------------------------------------------------------------- octree
// octree.cpp:7-51
int build_node(Scene& sc, BBox box, std::vector<std::pair<int, int>>& tris) {
    if (tris.empty()) return -1;
    if (tris.size() < 20) {
        Node nd;
        nd.box = box;
        nd.tris = tris;
        sc.nodes.push_back(std::move(nd));
        return (int)sc.nodes.size() - 1;
    }
    std::vector<std::pair<int, int>> lists[8];
    V3 c = box.center();
    for (int i = 0; i < 8; i++) {
        V3 k = box.corner(i);
        BBox sub;
        sub.mn = vmin(k, c);
        sub.mx = vmax(k, c);
        for (auto& mt : tris)
            if (sc.meshes[mt.first].tri_bbox(mt.second).overlaps(sub)) lists[i].push_back(mt);
        if (tris.size() == lists[i].size()) {
            Node nd;
            nd.box = box;
            nd.tris = tris;
            sc.nodes.push_back(std::move(nd));
            return (int)sc.nodes.size() - 1;
        }
    }
    int self = (int)sc.nodes.size();
    sc.nodes.emplace_back();
    sc.nodes[self].box = box;
    for (int i = 0; i < 8; i++) {
        BBox cb;
        for (auto& mt : lists[i]) cb.expand(sc.meshes[mt.first].tri_bbox(mt.second));
        cb.mn = cb.mn - V3(0.1f, 0.1f, 0.1f);
        int ch = build_node(sc, cb, lists[i]);
        sc.nodes[self].child[i] = ch;
    }
    return self;
}

// octree.cpp:53-110
bool closest(const Scene& sc, int node, Ray& ray, P2& uv, float& t, std::pair<int, int>& f) {
    if (node < 0) return false;
    const Node& nd = sc.nodes[node];
    if (!nd.box.hit(ray)) return false;
    if (!nd.tris.empty()) {
        bool hit = false;
        float u_, v_, t_;
        for (auto& mt : nd.tris) {
            if (sc.meshes[mt.first].intersect(mt.second, ray, u_, v_, t_)) {
                ray.maxt = t_;
                uv = P2{u_, v_};
                t = t_;
                f = mt;
                hit = true;
            }
        }
        return hit;
    }
    bool hit = false;
    float t_ = 0;
    P2 uv_{0, 0};
    std::pair<int, int> f_;
    float nearTs[8];
    int index[8];
    for (int i = 0; i < 8; i++) {
        if (nd.child[i] < 0) {
            nearTs[i] = kInf;
        } else {
            float nT, fT;
            sc.nodes[nd.child[i]].box.slab(ray, nT, fT);
            nearTs[i] = nT;
        }
        index[i] = i;
    }
    std::sort(index, index + 8, [&](int a, int b) -> bool { return nearTs[a] < nearTs[b]; });
    for (int idx : index) {
        if (ray.maxt < nearTs[idx]) continue;
        if (closest(sc, nd.child[idx], ray, uv_, t_, f_)) {
            ray.maxt = t_;
            uv = uv_;
            t = t_;
            f = f_;
            hit = true;
        }
    }
    return hit;
}

// octree.cpp:112-133
bool anyhit(const Scene& sc, int node, const Ray& ray) {
    if (node < 0) return false;
    const Node& nd = sc.nodes[node];
    if (!nd.box.hit(ray)) return false;
    if (!nd.tris.empty()) {
        float u_, v_, t_;
        for (auto& mt : nd.tris)
            if (sc.meshes[mt.first].intersect(mt.second, ray, u_, v_, t_)) return true;
        return false;
    }
    for (int i = 0; i < 8; i++)
        if (anyhit(sc, nd.child[i], ray)) return true;
    return false;
}

// Bilinear, wrap-addressed lookup at normalised (u, v) (a CUDA texture with
// linear filtering and wrap addressing, fp32 weights).
V3 tex_bilinear(const Texture& T, float u, float v) {
    const int W = T.w, H = T.h;
    if (!std::isfinite(u) || !std::isfinite(v)) return V3();
    u = u - std::floor(u);
    v = v - std::floor(v);
    float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    float fx = std::floor(x), fy = std::floor(y);
    float ax = x - fx, ay = y - fy;
    int x0 = (int)fx, y0 = (int)fy, x1 = x0 + 1, y1 = y0 + 1;
    if (x0 < 0) x0 += W;
    if (y0 < 0) y0 += H;
    if (x1 >= W) x1 -= W;
    if (y1 >= H) y1 -= H;
    auto tx = [&](int yy, int xx) { return ld3(&T.rgb[3 * ((size_t)yy * W + xx)]); };
    float bx = 1.f - ax, by = 1.f - ay;
    return tx(y0, x0) * (bx * by) + tx(y0, x1) * (ax * by) + tx(y1, x0) * (bx * ay) + tx(y1, x1) * (ax * ay);
}

// The hit record of face `face` of mesh `mi` at barycentrics uv, distance t
// (octree.cpp:186-212, with the OptiX shader's texture coordinates and
// normal / tangent maps).
void fill_hit(const Scene& sc, int mi, int face, P2 uv, float t, Hit& its) {
    const Mesh& m = sc.meshes[mi];
    its.uv = uv;
    its.t = t;
    its.mesh = mi;
    its.prim = m.prim_offset + face;
    V3 bary(1 - uv.x - uv.y, uv.x, uv.y);
    V3 p0 = m.pos(face, 0), p1 = m.pos(face, 1), p2 = m.pos(face, 2);
    its.p = bary.x * p0 + bary.y * p1 + bary.z * p2;
    if (!m.UV.empty()) {
        auto tc = [&](int k) {
            uint32_t p = m.F[3 * face + k];
            return P2{m.UV[2 * p], m.UV[2 * p + 1]};
        };
        P2 a = tc(0), b = tc(1), c = tc(2);
        its.uv = P2{bary.x * a.x + bary.y * b.x + bary.z * c.x,
                    bary.x * a.y + bary.y * b.y + bary.z * c.y};
    }
    its.geo = make_frame(normalized(cross(p1 - p0, p2 - p0)));
    if (!m.N.empty()) {
        // only the third normal term is normalised (octree.cpp:202-206)
        V3 n = bary.x * m.nrm(face, 0) + bary.y * m.nrm(face, 1) +
               bary.z * normalized(m.nrm(face, 2));
        its.sh = make_frame(n);
    } else {
        its.sh = its.geo;
    }
    its.tuv = P2{0.f, 0.f};
    its.tan = V3();
    const Material& mat = sc.mats[m.material];
    if (mat.has_tex) {
        // texture coordinates as the OptiX shader (shader_common.h:38-45);
        // world-space normal / tangent maps of aniso_ggx (62-64, 104-107)
        its.tuv = m.UV.empty() ? P2{0.f, 0.f} : its.uv;
        auto mapped = [&](int tx) {
            V3 c = tex_bilinear(sc.textures[tx], its.tuv.x, its.tuv.y);
            return normalized(V3(c.x * 2.f - 1.f, c.y * 2.f - 1.f, c.z * 2.f - 1.f));
        };
        if (mat.type == DL_MAT_ANISO_GGX && mat.tex[3] >= 0) its.sh.n = mapped(mat.tex[3]);
        if (mat.type == DL_MAT_ANISO_GGX && mat.tex[4] >= 0) its.tan = mapped(mat.tex[4]);
    }
}

// octree.cpp:153-212
bool ray_intersect(const Scene& sc, const Ray& ray_in, Hit& its) {
    Ray ray = ray_in;
    std::pair<int, int> f(-1, -1);
    P2 uv{0, 0};
    float t = 0;
    if (!closest(sc, sc.root, ray, uv, t, f)) return false;
    fill_hit(sc, f.first, f.second, uv, t, its);
    return true;
}

// The material at a hit with its textures looked up (diffuse.cu:15-20,
// aniso_ggx.cu:19-35).
Material material_at(const Scene& sc, const Hit& its) {
    Material m = sc.mats[sc.meshes[its.mesh].material];
    if (!m.has_tex) return m;
    if (m.tex[0] >= 0) m.albedo = tex_bilinear(sc.textures[m.tex[0]], its.tuv.x, its.tuv.y);
    if (m.type == DL_MAT_ANISO_GGX && m.tex[1] >= 0) m.specular = tex_bilinear(sc.textures[m.tex[1]], its.tuv.x, its.tuv.y);
    if (m.type == DL_MAT_ANISO_GGX && m.tex[2] >= 0) {
        V3 a = tex_bilinear(sc.textures[m.tex[2]], its.tuv.x, its.tuv.y);
        m.ax = a.x;
        m.ay = a.y;
    }
    return m;
}

inline bool occluded(const Scene& sc, const Ray& r) { return anyhit(sc, sc.root, r); }

// ------------------------------------------------------------------ BSDFs
struct BRec {
    V3 wi, wo;
    float eta = 1.f;
    int measure = kUnknown;
};

bool is_diffuse(const Material& m) {
    return m.type == DL_MAT_DIFFUSE || m.type == DL_MAT_MICROFACET || m.type == DL_MAT_ANISO_GGX;
}

// microfacet.cpp:35-44 (double arithmetic as written)
float beckmann_g1(V3 wv, V3 wh, float alpha) {
    float c = dot(wv, wh) / wv.z;
    if (c <= 0) return 0.0f;
    float b = (float)(1.0 / (double)(alpha * tan_theta(wv)));
    double bd = b;
    return b < 1.6 ? (float)((3.535 * bd + 2.181 * bd * bd) / (1 + 2.276 * bd + 2.577 * bd * bd))
                   : 1.0f;
}

// aniso_ggx.cu:9-15
float ggx_g1(V3 v, float ax, float ay) {
    if (v.z <= 0.0f) return 0.0f;
    V3 vv(v.x * ax, v.y * ay, v.z);
    return 2.0f * v.z / (v.z + length(vv));
}
// include/optix/math/wrap.h:54-64
float ggx_pdf(V3 m, float ax, float ay) {
    if (m.z <= 0) return 0;
    V3 h(m.x / ax, m.y / ay, m.z);
    float len2 = dot(h, h);
    return 1.f / (kPi * ax * ay * len2 * len2);
}
// include/optix/math/wrap.h:67-77
V3 square_to_ggx(P2 s, float ax, float ay) {
    float z1 = s.x, z2 = s.y;
    float x = ax * std::sqrt(z1) / std::sqrt(1 - z1) * std::cos(2 * kPi * z2);
    float y = ay * std::sqrt(z1) / std::sqrt(1 - z1) * std::sin(2 * kPi * z2);
    return normalized(V3(-x, -y, 1));
}

V3 bsdf_eval(const Material& m, const BRec& r) {
    switch (m.type) {
        case DL_MAT_DIFFUSE:
            if (r.measure != kSolidAngle || r.wi.z <= 0 || r.wo.z <= 0) return V3();
            return m.albedo * kInvPi;
        case DL_MAT_MICROFACET: {
            V3 wh = normalized(r.wi + r.wo);
            float D = beckmann_pdf(wh, m.ax);
            float F = fresnel(dot(r.wi, wh), m.ext_ior, m.int_ior);
            float G = beckmann_g1(r.wi, wh, m.ax) * beckmann_g1(r.wo, wh, m.ax);
            float deno = 1 / (4 * r.wi.z * r.wo.z);
            float spec = m.ks * D * F * G * deno;
            return m.albedo * kInvPi + V3(spec, spec, spec);
        }
        case DL_MAT_ANISO_GGX: {
            if (r.wi.z <= 0 || r.wo.z <= 0) return V3();
            V3 wh = normalized(r.wi + r.wo);
            float D = ggx_pdf(wh, m.ax, m.ay);
            const float F0 = 0.04f;
            float ldoth = dot(r.wi, wh);
            float temp = std::fmin(std::fmax(0.0f, 1.0f - ldoth), 1.0f);
            float F = F0 + (1.0f - F0) * temp * temp * temp * temp * temp;
            float G = ggx_g1(r.wi, m.ax, m.ay) * ggx_g1(r.wo, m.ax, m.ay);
            float deno = 1.f / (4.f * r.wi.z * r.wo.z);
            return m.albedo * kInvPi + m.specular * D * F * G * deno;
        }
        default:
            return V3();  // mirror, dielectric: discrete
    }
}

float bsdf_pdf(const Material& m, const BRec& r) {
    switch (m.type) {
        case DL_MAT_DIFFUSE:
            if (r.measure != kSolidAngle || r.wi.z <= 0 || r.wo.z <= 0) return 0.0f;
            return kInvPi * r.wo.z;
        case DL_MAT_MICROFACET: {
            if (r.measure != kSolidAngle || r.wi.z <= 0 || r.wo.z <= 0) return 0.0f;
            V3 wh = normalized(r.wi + r.wo);
            float diff = (1 - m.ks) * cosine_hemisphere_pdf(r.wo);
            float spec = m.ks * beckmann_pdf(wh, m.ax) / 4 / dot(wh, r.wo);
            return diff + spec;
        }
        case DL_MAT_ANISO_GGX: {
            if (r.measure != kSolidAngle || r.wi.z <= 0 || r.wo.z <= 0) return 0.f;
            V3 wh = normalized(r.wi + r.wo);
            float diff = (1 - 0.5f) * cosine_hemisphere_pdf(r.wo);
            float spec = 0.5f * ggx_pdf(wh, m.ax, m.ay) * wh.z / 4.f / dot(wh, r.wo);
            return diff + spec;
        }
        default:
            return 0.0f;
    }
}

// `lobe` is the third uniform number of aniso_ggx's sample (aniso_ggx.cu:
// 104-108: drawn after the 2D sample, > 0.5 picks the diffuse lobe); the
// other materials ignore it.
V3 bsdf_sample(const Material& m, BRec& r, P2 s, float lobe) {
    switch (m.type) {
        case DL_MAT_DIFFUSE:
            if (r.wi.z <= 0) return V3();
            r.measure = kSolidAngle;
            r.wo = square_to_cosine_hemisphere(s);
            r.eta = 1.0f;
            return m.albedo;
        case DL_MAT_MIRROR:
            if (r.wi.z <= 0) return V3();
            r.wo = V3(-r.wi.x, -r.wi.y, r.wi.z);
            r.measure = kDiscrete;
            r.eta = 1.0f;
            return V3(1.0f, 1.0f, 1.0f);
        case DL_MAT_DIELECTRIC: {
            r.measure = kDiscrete;
            float cosI = r.wi.z;
            float ri = fresnel(cosI, m.ext_ior, m.int_ior);
            if (s.x < ri) {
                r.wo = V3(-r.wi.x, -r.wi.y, r.wi.z);
                r.eta = 1;
            } else {
                float eta = m.ext_ior / m.int_ior;
                r.wo = normalized(refract(r.wi, eta));
                r.eta = cosI > 0.f ? eta : 1 / eta;
            }
            return V3(1.f, 1.f, 1.f);
        }
        case DL_MAT_MICROFACET: {
            if (r.wi.z <= 0) return V3();
            r.measure = kSolidAngle;
            float sx = s.x;
            P2 ss = s;
            if (sx > m.ks) {
                ss.x = (sx - m.ks) / (1 - m.ks);
                r.wo = square_to_cosine_hemisphere(ss);
            } else {
                ss.x = sx / m.ks;
                V3 wh = square_to_beckmann(ss, m.ax);
                r.wo = reflect(r.wi, wh);
            }
            if (r.wo.z <= 0) return V3();
            return bsdf_eval(m, r) * r.wo.z / bsdf_pdf(m, r);
        }
        case DL_MAT_ANISO_GGX: {
            // aniso_ggx.cu:89-121: the third number picks the lobe, the 2D
            // sample drives it unchanged
            if (r.wi.z <= 0) return V3();
            r.measure = kSolidAngle;
            if (lobe > 0.5f) {
                r.wo = square_to_cosine_hemisphere(s);
            } else {
                V3 wh = square_to_ggx(s, m.ax, m.ay);
                r.wo = reflect(r.wi, wh);
            }
            if (r.wo.z <= 0) return V3();
            return bsdf_eval(m, r) * r.wo.z / bsdf_pdf(m, r);
        }
        default:
            return V3();
    }
}

// ---------------------------------------------------------------- emitters
struct DirSample {
    V3 o, d, n;
    float dist = 0, pdf = 0;
};
inline DirSample make_ds(V3 o, V3 dst, V3 n) {
    DirSample ds;
    ds.o = o;
    ds.n = n;
    V3 vec = dst - o;
    ds.d = normalized(vec);
    ds.dist = length(vec);
    return ds;
}

// area.cpp:11-37, point.cpp:17-25 (+ the OptiX cosine when fixed)
V3 emitter_sample_direction(const Scene& sc, const Light& L, P2 s, const Hit& its, DirSample& ds,
                            uint32_t flags) {
    if (L.type == DL_LIGHT_AREA) {
        const Mesh& m = sc.meshes[L.mesh];
        V3 p, n;
        m.sample_position(s, p, n);
        ds = make_ds(its.p, p, n);
        float pA = m.dpdf.norm;
        float dp = std::max(dot(n, -ds.d), 0.0f);
        float pw = dp != 0 ? pA * ds.dist * ds.dist / dp : 0;
        ds.pdf = pw;
        if (pw == 0) return V3();
        float c = std::max(dot(its.sh.n, ds.d), 0.0f);
        return L.radiance * c / pw;
    }
    if (L.type == DL_LIGHT_POINT) {
        ds = make_ds(its.p, L.position, V3(0.f, 0.f, 0.f));
        ds.pdf = 1;
        float inv = (float)(1.0 / (double)ds.dist);
        if (flags & DL_RENDER_FIX_POINT_LIGHT) {
            float c = std::fmax(dot(its.sh.n, ds.d), 0.f);
            return c > 0.f ? L.radiance * c * inv * inv : V3();
        }
        return L.radiance * inv * inv;
    }
    ds.pdf = 0;
    return V3();
}

// ---------------------------------------------------------------- envmap
// The envmap emitter exists only in the reference's OptiX backend
// (include/optix/light/envmap.h:25-94, tables from src/tracer/emitter/
// envmap.cpp:59-141; miss shading src/optix/cuda/miss.cu:11-49).  Restated
// here with the C float functions for CUDA's atan2f/acosf/cosf/sinf, a
// bilinear, wrap-addressed lookup for the reference's linear-filtered float
// texture, and the pcg32 ordering of this renderer: an envmap pick in NEE
// draws three fresh numbers after the NEE 2D sample.

// envmap.cpp:59-141 (importance, alias table, pdf)
void env_build(Light& L) {
    const uint32_t rx = L.env_w, ry = L.env_h, size = rx * ry;
    const float* px = L.env_rgb.data();
    std::vector<float> imp(size);
    L.env_q.assign(size, 0.f);
    L.env_pdf.assign(size, 0.f);
    L.env_alias.assign(size, 0u);
    auto maxc3 = [&](uint32_t i) { return std::max(px[3 * i], std::max(px[3 * i + 1], px[3 * i + 2])); };
    float cos_theta0 = 1.0f;
    const float step_phi = (float)(2.0 * (double)kPi) / (float)rx;
    const float step_theta = kPi / (float)ry;
    for (uint32_t y = 0; y < ry; ++y) {
        const float theta1 = (float)(y + 1) * step_theta;
        const float cos_theta1 = (float)std::cos((double)theta1);
        const float area = (cos_theta0 - cos_theta1) * step_phi;
        cos_theta0 = cos_theta1;
        for (uint32_t x = 0; x < rx; ++x) imp[y * rx + x] = area * maxc3(y * rx + x);
    }
    // sum and residual chain in double (the renderer's choice: the
    // reference's float chain misstates pick probabilities on bright suns)
    double sum = 0.0;
    for (uint32_t i = 0; i < size; ++i) sum += imp[i];
    if (!(sum > 0.0)) {
        for (uint32_t i = 0; i < size; ++i) {
            L.env_q[i] = 1.0f;
            L.env_alias[i] = i;
        }
        return;
    }
    L.env_sum = sum;
    std::vector<double> q(size);
    for (uint32_t i = 0; i < size; ++i) q[i] = (double)size * imp[i] / sum;
    std::vector<uint32_t> part(size);
    uint32_t s = 0u, large = size;
    for (uint32_t i = 0; i < size; ++i) part[(q[i] < 1.0) ? (s++) : (--large)] = L.env_alias[i] = i;
    for (s = 0; s < large && large < size; ++s) {
        const uint32_t j = part[s], k = part[large];
        L.env_alias[j] = k;
        q[k] += q[j] - 1.0;
        large = (q[k] < 1.0) ? (large + 1u) : large;
    }
    for (uint32_t i = 0; i < size; ++i) {
        L.env_q[i] = (float)q[i];
        L.env_pdf[i] = (float)((double)maxc3(i) / sum);
    }
}

// linear filter, wrap addressing, normalised coordinates
V3 env_lookup(const Light& L, float u, float v) {
    const int W = L.env_w, H = L.env_h;
    if (!std::isfinite(u) || !std::isfinite(v)) return V3();  // no direction
    u = u - std::floor(u);
    v = v - std::floor(v);
    float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    float fx = std::floor(x), fy = std::floor(y);
    float ax = x - fx, ay = y - fy;
    int x0 = (int)fx, y0 = (int)fy, x1 = x0 + 1, y1 = y0 + 1;
    if (x0 < 0) x0 += W;
    if (y0 < 0) y0 += H;
    if (x1 >= W) x1 -= W;
    if (y1 >= H) y1 -= H;
    auto tx = [&](int yy, int xx) { return ld3(&L.env_rgb[3 * ((size_t)yy * W + xx)]); };
    float bx = 1.f - ax, by = 1.f - ay;
    V3 r = tx(y0, x0) * (bx * by) + tx(y0, x1) * (ax * by) + tx(y1, x0) * (bx * ay) + tx(y1, x1) * (ax * ay);
    return r * L.env_scale;
}

// envmap.h:26-30
P2 env_coords(V3 d) {
    float u = std::atan2(d.z, d.x) * (float)(0.5 / (double)kPi) + 0.5f;
    float v = std::acos(std::fmax(std::fmin(d.y, 1.0f), -1.0f)) * kInvPi;
    return P2{u, v};
}

V3 env_eval(const Light& L, V3 d) {
    P2 uv = env_coords(d);
    return env_lookup(L, uv.x, uv.y);
}

// envmap.h:78-84
float env_pdf(const Light& L, V3 d) {
    P2 uv = env_coords(d);
    int x = std::min((int)(uv.x * (float)L.env_w), L.env_w - 1);
    int y = std::min((int)(uv.y * (float)L.env_h), L.env_h - 1);
    return L.env_pdf[(size_t)y * L.env_w + x];
}

// envmap.h:33-76
V3 env_sample(const Light& L, const Hit& its, V3 xi, DirSample& ds) {
    const uint32_t W = L.env_w, H = L.env_h, size = W * H;
    uint32_t idx = std::min((uint32_t)(xi.x * (float)size), size - 1);
    uint32_t env_idx;
    float xy = xi.y;
    if (xy < L.env_q[idx]) {
        env_idx = idx;
        xy /= L.env_q[idx];
    } else {
        env_idx = L.env_alias[idx];
        xy = (xy - L.env_q[idx]) / (1.0f - L.env_q[idx]);
    }
    const uint32_t py = env_idx / W, px = env_idx % W;
    float pdf = L.env_pdf[env_idx];
    float u = ((float)px + xy) / (float)W;
    float phi = (float)((double)u * 2.0 * (double)kPi - (double)kPi);
    float step_theta = kPi / (float)H;
    float theta0 = (float)py * step_theta;
    float cos_theta = std::cos(theta0) * (1.0f - xi.z) + std::cos(theta0 + step_theta) * xi.z;
    float theta = std::acos(cos_theta);
    float sin_theta = std::sin(theta);
    ds.o = its.p;
    ds.d = V3(std::cos(phi) * sin_theta, cos_theta, std::sin(phi) * sin_theta);
    ds.n = -ds.d;
    ds.dist = 1e16f;
    ds.pdf = pdf;
    if (!(pdf > 0.f)) return V3();
    V3 val = env_lookup(L, u, theta * kInvPi);
    float c = std::max(dot(its.sh.n, ds.d), 0.f);
    return c > 0.f ? val * c / pdf : V3();
}

float emitter_pdf_direction(const Scene& sc, const Light& L, const DirSample& ds) {
    if (L.type == DL_LIGHT_AREA) {
        float pA = sc.meshes[L.mesh].dpdf.norm;
        float dp = std::max(dot(ds.n, -ds.d), 0.0f);
        return dp != 0 ? pA * ds.dist * ds.dist / dp : 0;
    }
    if (L.type == DL_LIGHT_ENVMAP) return env_pdf(L, ds.d);
    return 0;
}

// scene.cpp:139-170; `delta` reports a point light (for the fix flag).  An
// envmap pick draws three numbers from `rng` (none given: no sample).
void sample_emitter(const Scene& sc, const Hit& its, P2 s, DirSample& ds, V3& spec, bool& delta,
                    uint32_t flags, Pcg32* rng) {
    size_t N = sc.lights.size();
    delta = false;
    auto one = [&](const Light& L, P2 ss) {
        if (L.type != DL_LIGHT_ENVMAP) return emitter_sample_direction(sc, L, ss, its, ds, flags);
        if (!rng) {
            ds.pdf = 0;
            return V3();
        }
        V3 xi;
        xi.x = rng->next1d();
        xi.y = rng->next1d();
        xi.z = rng->next1d();
        return env_sample(L, its, xi, ds);
    };
    if (N == 0) {
        spec = V3();
    } else if (flags & DL_RENDER_POWER_LIGHT_PICK) {
        // alias pick: slot from s.x * N, coin from its fraction, reused
        float u = s.x * (float)N;
        size_t i = std::min((size_t)u, N - 1);
        float coin = std::fmin(u - (float)i, 0.99999994f);
        size_t idx = i;
        if (coin < sc.pick_q[i]) {
            s.x = coin / sc.pick_q[i];
        } else {
            s.x = (coin - sc.pick_q[i]) / (1.f - sc.pick_q[i]);
            idx = sc.pick_alias[i];
        }
        const float pl = sc.pick_prob[idx];
        spec = one(sc.lights[idx], s);
        delta = sc.lights[idx].type == DL_LIGHT_POINT;
        spec = spec / pl;
        ds.pdf *= pl;
    } else if (N == 1) {
        spec = one(sc.lights[0], s);
        delta = sc.lights[0].type == DL_LIGHT_POINT;
    } else {
        float epdf = 1.f / N;
        size_t idx = std::min((size_t)(s.x * N), N - 1);
        s.x = s.x * N - idx;
        spec = one(sc.lights[idx], s);
        delta = sc.lights[idx].type == DL_LIGHT_POINT;
        spec = spec * (float)N;
        ds.pdf *= epdf;
    }
    if (spec.x + spec.y + spec.z > 0) {
        Ray r = make_ray(its.p, ds.d, kEps, ds.dist - kEps);
        spec = spec * (1 - (float)occluded(sc, r));
    }
}

float pdf_emitter(const Scene& sc, int light, const DirSample& ds, uint32_t flags) {
    if (flags & DL_RENDER_POWER_LIGHT_PICK) return emitter_pdf_direction(sc, sc.lights[light], ds) * sc.pick_prob[light];
    if (sc.lights.size() == 1) return emitter_pdf_direction(sc, sc.lights[0], ds);
    return emitter_pdf_direction(sc, sc.lights[light], ds) / sc.lights.size();
}

inline float mis(float a, float b) {
    a *= a;
    b *= b;
    return a / (a + b);
}

// __miss__radiance (miss.cu:11-49) of a ray leaving along d: a camera ray
// sees the envmap if "visual", else the background colour (weight 1); a
// later ray gets the envmap's radiance with weight w, the MIS weight against
// the pdf of the BSDF sample that made it when that BSDF is diffuse, else 1.
V3 env_miss(const Scene& sc, V3 d, bool camera, bool diffuse, float bsdf_pdf, uint32_t flags, float& w) {
    const Light& E = sc.lights[sc.env_light];
    w = 1.f;
    if (camera) return E.env_visual ? env_eval(E, d) : E.env_bg;
    if (diffuse) {
        DirSample hs;
        hs.d = d;
        w = mis(bsdf_pdf, pdf_emitter(sc, sc.env_light, hs, flags));
    }
    return env_eval(E, d);
}

inline V3 emitter_eval(const Light& L, const Hit& its, V3 wi) {
    if (L.type != DL_LIGHT_AREA) return V3();
    float c = to_local(its.sh, wi).z;
    return c > 0.f ? L.radiance : V3();
}

// Local shading frame of a hit for a material (Nori frame; the OptiX Onb
// for aniso_ggx).
inline Frame shading_frame(const Scene& sc, const Hit& its) {
    const Material& m = sc.mats[sc.meshes[its.mesh].material];
    if (m.type == DL_MAT_ANISO_GGX) return make_onb_t(normalized(its.sh.n), its.tan);
    return its.sh;
}

struct Opts {
    int max_depth = 0;
    int rr_depth = 3;
    uint32_t flags = 0;
};

// path.cpp:13-100 (+ max_depth and rr_depth options; reference: 0 and 3)
V3 Li(const Scene& sc, Pcg32& rng, const Ray& ray_in, const Opts& o) {
    Ray ray = ray_in;
    float eta = 1.f;
    V3 result, tp(1.f, 1.f, 1.f);
    Hit its;
    if (o.flags & DL_RENDER_NORMALS) {
        // normal.cpp:10-20: |shading normal| of the first hit, 0 on a miss
        if (!ray_intersect(sc, ray, its)) return result;
        return V3(std::fabs(its.sh.n.x), std::fabs(its.sh.n.y), std::fabs(its.sh.n.z));
    }
    if (!ray_intersect(sc, ray, its)) {
        // miss.cu:20-27: the camera sees the envmap if "visual", else bg_color
        float w;
        if (sc.env_light >= 0) result = env_miss(sc, ray.d, true, false, 0.f, o.flags, w);
        return result;
    }
    int light = sc.meshes[its.mesh].light;
    if (light >= 0) result = result + mul(tp, emitter_eval(sc.lights[light], its, -ray.d));
    for (int depth = 0;; ++depth) {
        if (o.max_depth > 0 && depth >= o.max_depth) break;
        const Material bsdf = material_at(sc, its);
        Frame fr = shading_frame(sc, its);
        DirSample ds;
        V3 ev;
        bool delta = false;
        sample_emitter(sc, its, rng.next2d(), ds, ev, delta, o.flags, &rng);
        V3 wi = to_local(fr, -normalized(ray.d));
        if (bsdf.type == DL_MAT_ANISO_GGX) wi = normalized(wi);
        V3 wo = to_local(fr, ds.d);
        BRec q;
        q.wi = wi;
        q.wo = wo;
        q.measure = kSolidAngle;
        if (ds.pdf > 0) {
            V3 bv = bsdf_eval(bsdf, q);
            float bp = bsdf_pdf(bsdf, q);
            float w = (delta && (o.flags & DL_RENDER_FIX_POINT_LIGHT)) ? 1.f : mis(ds.pdf, bp);
            result = result + mul(mul(w * tp, bv), ev);
        }
        BRec bq;
        bq.wi = wi;
        const P2 s2 = rng.next2d();
        const float lobe = bsdf.type == DL_MAT_ANISO_GGX ? rng.next1d() : 0.f;
        V3 f = bsdf_sample(bsdf, bq, s2, lobe);
        tp = mul(tp, f);
        eta *= bq.eta;
        V3 nd = to_world(fr, bq.wo);
        if (bsdf.type == DL_MAT_ANISO_GGX) nd = normalized(nd);
        ray = make_ray(its.p, nd);
        if (ray_intersect(sc, ray, its)) {
            int lt = sc.meshes[its.mesh].light;
            if (lt >= 0) {
                V3 le = emitter_eval(sc.lights[lt], its, -ray.d);
                DirSample hs = make_ds(ray.o, its.p, its.sh.n);
                float ep = pdf_emitter(sc, lt, hs, o.flags);
                float bp = bsdf_pdf(bsdf, bq);
                float w = is_diffuse(bsdf) ? mis(bp, ep) : 1.f;
                result = result + mul(w * tp, le);
            }
        } else {
            // miss.cu:28-44: envmap radiance, MIS-weighted after a diffuse
            // bounce (a path with zero throughput adds nothing)
            if (sc.env_light >= 0 && (tp.x != 0.f || tp.y != 0.f || tp.z != 0.f)) {
                const float bp = is_diffuse(bsdf) ? bsdf_pdf(bsdf, bq) : 0.f;
                float w;
                V3 le = env_miss(sc, ray.d, false, is_diffuse(bsdf), bp, o.flags, w);
                result = result + mul(w * tp, le);
            }
            break;
        }
        if (depth > o.rr_depth) {
            float p = std::min(maxc(tp * eta * eta), (float)0.99);
            if (rng.next1d() > p) break;
            tp = tp / p;
        }
    }
    return result;
}

// --------------------------------------------------------------- camera
static void camera_matrices(const dl_camera_desc& c, Camera& cam);

// virtual.cpp:16-42
Camera make_camera(const dl_camera_desc& c) {
    Camera cam;
    cam.w = c.width;
    cam.h = c.height;
    cam.inv_w = 1.f / c.width;
    cam.inv_h = 1.f / c.height;
    if (c.type != DL_CAMERA_VIRTUAL) {
        camera_matrices(c, cam);
        return cam;
    }
    float fov = c.fov;
    float aspect = c.width / (float)c.height;
    V3 eye = ld3(c.eye), look = ld3(c.lookat), up = ld3(c.up);
    cam.W = look - eye;
    float wlen = length(cam.W);
    cam.U = normalized(cross(cam.W, up));
    cam.V = normalized(cross(cam.U, cam.W));
    float vlen = wlen * tanf(0.5f * fov * kPi / 180.f);
    cam.V = cam.V * vlen;
    float ulen = vlen * aspect;
    cam.U = cam.U * ulen;
    cam.eye = eye;
    return cam;
}
// Inverse of a 4x4 matrix given in double, rounded to float: reduce [A | I]
// to [I | A^-1] with the largest remaining entry as pivot.
static bool oracle_inverse4(const double* a, float* out) {
    double m[4][4], r[4][4];
    int col[4] = {0, 1, 2, 3}, row[4] = {0, 1, 2, 3};
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            m[i][j] = a[4 * i + j];
            r[i][j] = i == j ? 1.0 : 0.0;
        }
    for (int k = 0; k < 4; k++) {
        int pr = k;
        for (int i = k + 1; i < 4; i++)
            if (std::fabs(m[i][k]) > std::fabs(m[pr][k])) pr = i;
        if (!(std::fabs(m[pr][k]) > 1e-30)) return false;
        for (int j = 0; j < 4; j++) {
            std::swap(m[k][j], m[pr][j]);
            std::swap(r[k][j], r[pr][j]);
        }
        const double p = m[k][k];
        for (int j = 0; j < 4; j++) {
            m[k][j] /= p;
            r[k][j] /= p;
        }
        for (int i = 0; i < 4; i++) {
            if (i == k) continue;
            const double f = m[i][k];
            for (int j = 0; j < 4; j++) {
                m[i][j] -= f * m[k][j];
                r[i][j] -= f * r[k][j];
            }
        }
    }
    (void)col;
    (void)row;
    for (int i = 0; i < 16; i++) out[i] = (float)r[i / 4][i % 4];
    return true;
}

// perspective.cpp:41-73 (the sample-to-camera matrix = (scale * translate *
// projection)^-1, here in double); opencv.cpp:10-24 (inverse extrinsic, eye).
static void camera_matrices(const dl_camera_desc& c, Camera& cam) {
    cam.type = c.type;
    if (c.type == DL_CAMERA_PERSPECTIVE) {
        const double aspect = (double)(c.width / (float)c.height);
        const double n = c.near_clip, f = c.far_clip;
        const double cot = 1.0 / std::tan((double)c.fov / 2.0 * (3.14159265358979323846 / 180.0));
        const double recip = 1.0 / (f - n);
        // scale(-1/2, -aspect/2, 1) * translate(-1, -1/aspect, 0) * projection
        double proj[4][4] = {{cot, 0, 0, 0}, {0, cot, 0, 0}, {0, 0, f * recip, -n * f * recip}, {0, 0, 1, 0}};
        const double sx = -0.5, sy = -0.5 * aspect, tx = -1.0, ty = -1.0 / aspect;
        double M[16];
        for (int j = 0; j < 4; j++) {
            M[0 * 4 + j] = sx * (proj[0][j] + tx * proj[3][j]);
            M[1 * 4 + j] = sy * (proj[1][j] + ty * proj[3][j]);
            M[2 * 4 + j] = proj[2][j];
            M[3 * 4 + j] = proj[3][j];
        }
        if (!oracle_inverse4(M, cam.S)) throw std::runtime_error("singular perspective projection");
        for (int k = 0; k < 16; k++) cam.T[k] = c.transform[k];
        cam.far_clip = c.far_clip;
    } else if (c.type == DL_CAMERA_OPENCV) {
        double E[16];
        for (int k = 0; k < 16; k++) E[k] = c.transform[k];
        if (!oracle_inverse4(E, cam.T)) throw std::runtime_error("singular extrinsic");
        cam.eye = V3(cam.T[3], cam.T[7], cam.T[11]);
        cam.fx = c.fx;
        cam.fy = c.fy;
        cam.cx = c.cx;
        cam.cy = c.cy;
    }
}

// Matrix4f * Vector4f, row i (include/core/math/matrix.h:265-271 and
// TVector::dot: a running sum from 0, left to right).
static float mat_row(const float* m, int i, float a0, float a1, float a2, float a3) {
    float sum = 0.f;
    sum += a0 * m[4 * i];
    sum += a1 * m[4 * i + 1];
    sum += a2 * m[4 * i + 2];
    sum += a3 * m[4 * i + 3];
    return sum;
}

// virtual.cpp:52-65; perspective.cpp:84-100; include/optix/camera/opencv.h:
// 29-46 with the film position as the pixel sample.  Render rays start at
// kEps; the perspective camera's far end is far / d.z.
Ray camera_ray(const Camera& c, P2 s) {
    if (c.type == DL_CAMERA_PERSPECTIVE) {
        const float sx = s.x * c.inv_w, sy = s.y * c.inv_h;
        const float w = mat_row(c.S, 3, sx, sy, 0.f, 1.f);
        const V3 nearP(mat_row(c.S, 0, sx, sy, 0.f, 1.f) / w, mat_row(c.S, 1, sx, sy, 0.f, 1.f) / w,
                       mat_row(c.S, 2, sx, sy, 0.f, 1.f) / w);
        float sum = 0.f;
        sum += nearP.x * nearP.x;
        sum += nearP.y * nearP.y;
        sum += nearP.z * nearP.z;
        const float len = std::sqrt(sum);
        const V3 d(nearP.x / len, nearP.y / len, nearP.z / len);
        const float invZ = 1.0f / d.z;
        const float ow = mat_row(c.T, 3, 0.f, 0.f, 0.f, 1.f);
        const V3 o(mat_row(c.T, 0, 0.f, 0.f, 0.f, 1.f) / ow, mat_row(c.T, 1, 0.f, 0.f, 0.f, 1.f) / ow,
                   mat_row(c.T, 2, 0.f, 0.f, 0.f, 1.f) / ow);
        const V3 dw(mat_row(c.T, 0, d.x, d.y, d.z, 0.f), mat_row(c.T, 1, d.x, d.y, d.z, 0.f),
                    mat_row(c.T, 2, d.x, d.y, d.z, 0.f));
        return make_ray(o, dw, kEps, c.far_clip * invZ);
    }
    if (c.type == DL_CAMERA_OPENCV) {
        const float px = (s.x - c.cx) / c.fx, py = (s.y - c.cy) / c.fy;
        const V3 head(mat_row(c.T, 0, px, py, 1.f, 1.f), mat_row(c.T, 1, px, py, 1.f, 1.f),
                      mat_row(c.T, 2, px, py, 1.f, 1.f));
        return make_ray(c.eye, normalized(head - c.eye));
    }
    float lx = s.x, ly = (float)c.h - s.y - 1;
    float px = lx * c.inv_w * 2 - 1, py = ly * c.inv_h * 2 - 1;
    V3 d = normalized(px * c.U + py * c.V + c.W);
    return make_ray(c.eye, d);
}

// ----------------------------------------------------------------- film
// rfilter.cpp + block.cpp:10-28
Filter make_filter(int kind) {
    Filter f;
    const int RES = 32;
    if (kind == DL_FILTER_BOX) {
        f.radius = 0.5f;
    } else {
        f.radius = 2.0f;
    }
    f.border = (int)std::ceil(f.radius - 0.5f);
    for (int i = 0; i < RES; ++i) {
        float pos = (f.radius * i) / RES;
        if (kind == DL_FILTER_BOX) {
            f.table[i] = 1.0f;
        } else {
            const float stddev = 0.5f;
            float alpha = -1.0f / (2.0f * stddev * stddev);
            f.table[i] = std::max(0.0f, std::exp(alpha * pos * pos) -
                                            std::exp(alpha * f.radius * f.radius));
        }
    }
    f.table[RES] = 0.0f;
    f.lookup = RES / f.radius;
    return f;
}

struct Film {
    int ox = 0, oy = 0;  // offset of the block in the image
    int w = 0, h = 0;    // block size without border
    int b = 0;
    std::vector<float> px;  // (h+2b) x (w+2b) x 4
    int cols() const { return w + 2 * b; }
    int rows() const { return h + 2 * b; }
    void reset(int x, int y, int ww, int hh, int border) {
        ox = x; oy = y; w = ww; h = hh; b = border;
        px.assign((size_t)cols() * rows() * 4, 0.f);
    }
};

inline bool valid(V3 c) {
    for (int i = 0; i < 3; i++) {
        float v = c[i];
        if (v < 0 || !std::isfinite(v)) return false;
    }
    return true;
}

// block.cpp:81-113
bool film_put(Film& fb, const Filter& F, P2 pos_in, V3 value) {
    if (!valid(value)) return false;
    float px = pos_in.x - 0.5f - (float)(fb.ox - fb.b);
    float py = pos_in.y - 0.5f - (float)(fb.oy - fb.b);
    int x0 = (int)std::ceil(px - F.radius), y0 = (int)std::ceil(py - F.radius);
    int x1 = (int)std::floor(px + F.radius), y1 = (int)std::floor(py + F.radius);
    x0 = std::max(x0, 0);
    y0 = std::max(y0, 0);
    x1 = std::min(x1, fb.cols() - 1);
    y1 = std::min(y1, fb.rows() - 1);
    float wx[8], wy[8];
    for (int x = x0, i = 0; x <= x1; ++x) wx[i++] = F.table[(int)(std::abs(x - px) * F.lookup)];
    for (int y = y0, i = 0; y <= y1; ++y) wy[i++] = F.table[(int)(std::abs(y - py) * F.lookup)];
    for (int y = y0, yr = 0; y <= y1; ++y, ++yr)
        for (int x = x0, xr = 0; x <= x1; ++x, ++xr) {
            float* c = &fb.px[((size_t)y * fb.cols() + x) * 4];
            c[0] += value.x * wx[xr] * wy[yr];
            c[1] += value.y * wx[xr] * wy[yr];
            c[2] += value.z * wx[xr] * wy[yr];
            c[3] += 1.0f * wx[xr] * wy[yr];
        }
    return true;
}

// block.cpp:115-129
void film_merge(Film& dst, const Film& src) {
    int offx = src.ox - dst.ox + (dst.b - src.b);
    int offy = src.oy - dst.oy + (dst.b - src.b);
    int sw = src.cols(), sh = src.rows();
    for (int i = 0; i < sh; i++)
        for (int j = 0; j < sw; j++) {
            float* d = &dst.px[((size_t)(offy + i) * dst.cols() + (offx + j)) * 4];
            const float* s = &src.px[((size_t)i * sw + j) * 4];
            for (int k = 0; k < 4; k++) d[k] += s[k];
        }
}

void film_outputs(const Film& fb, float* rgb, float* film) {
    if (rgb)
        for (int y = 0; y < fb.h; y++)
            for (int x = 0; x < fb.w; x++) {
                const float* c = &fb.px[((size_t)(y + fb.b) * fb.cols() + (x + fb.b)) * 4];
                float* o = rgb + 3 * ((size_t)y * fb.w + x);
                if (c[3] != 0) {
                    o[0] = c[0] / c[3]; o[1] = c[1] / c[3]; o[2] = c[2] / c[3];
                } else {
                    o[0] = o[1] = o[2] = 0.f;
                }
            }
    if (film) std::memcpy(film, fb.px.data(), fb.px.size() * sizeof(float));
}

// block.cpp:131-177: spiral order of 32x32 blocks from the image centre.
std::vector<std::pair<int, int>> spiral_blocks(int w, int h, int bs) {
    int nx = (int)std::ceil(w / (float)bs), ny = (int)std::ceil(h / (float)bs);
    int left = nx * ny;
    int dir = 0;  // right, down, left, up
    int bx = nx / 2, by = ny / 2;
    int steps_left = 1, num_steps = 1;
    std::vector<std::pair<int, int>> out;
    while (left > 0) {
        out.push_back({bx * bs, by * bs});
        if (--left == 0) break;
        do {
            switch (dir) {
                case 0: ++bx; break;
                case 1: ++by; break;
                case 2: --bx; break;
                case 3: --by; break;
            }
            if (--steps_left == 0) {
                dir = (dir + 1) % 4;
                if (dir == 2 || dir == 0) ++num_steps;
                steps_left = num_steps;
            }
        } while (bx < 0 || by < 0 || bx >= nx || by >= ny);
    }
    return out;
}

Opts opts_of(const dl_render_opts* o) {
    Opts r;
    if (o) {
        r.max_depth = o->max_depth;
        r.rr_depth = o->rr_depth;
        r.flags = o->flags;
    }
    return r;
}

inline void seed_path(Pcg32& rng, uint64_t seed, int w, int h, int x, int y, int s) {
    uint64_t seq = (uint64_t)s * (uint64_t)w * (uint64_t)h + (uint64_t)y * (uint64_t)w + (uint64_t)x;
    rng.seed(splitmix64(seq ^ splitmix64(seed)), seq);
}

template <typename F>
void parallel(int threads, int64_t n, F fn) {
    int T = std::max(1, threads);
    std::vector<std::thread> th;
    for (int k = 0; k < T; k++) th.emplace_back([&, k] { fn(k, n * k / T, n * (k + 1) / T); });
    for (auto& t : th) t.join();
}

}  // namespace

extern "C" {

const char* orc_last_error(void) { return g_error.c_str(); }

void* orc_scene_create(const dl_mesh_desc* meshes, int32_t nm, const dl_material_desc* mats,
                       int32_t nmat, const dl_light_desc* lights, int32_t nl,
                       const dl_camera_desc* cam, int32_t filter) {
    auto* sc = new Scene();
    for (int i = 0; i < nmat; i++) {
        Material m;
        m.type = mats[i].type;
        m.albedo = ld3(mats[i].albedo);
        m.specular = ld3(mats[i].specular);
        m.ax = mats[i].alpha[0];
        m.ay = mats[i].alpha[1];
        m.int_ior = mats[i].int_ior;
        m.ext_ior = mats[i].ext_ior;
        m.ks = 1 - maxc(m.albedo);
        const dl_texture_desc* slots[5] = {&mats[i].albedo_texture, &mats[i].specular_texture,
                                           &mats[i].alpha_texture, &mats[i].normal_texture,
                                           &mats[i].tangent_texture};
        for (int k = 0; k < 5; k++) {
            if (!slots[k]->rgb) continue;
            Texture t;
            t.w = slots[k]->width;
            t.h = slots[k]->height;
            t.rgb.assign(slots[k]->rgb, slots[k]->rgb + 3 * (size_t)t.w * t.h);
            m.tex[k] = (int)sc->textures.size();
            sc->textures.push_back(std::move(t));
            m.has_tex = true;
        }
        sc->mats.push_back(m);
    }
    int64_t off = 0;
    for (int i = 0; i < nm; i++) {
        const dl_mesh_desc& d = meshes[i];
        Mesh m;
        m.V.assign(d.positions, d.positions + 3 * d.num_vertices);
        if (d.normals) m.N.assign(d.normals, d.normals + 3 * d.num_vertices);
        if (d.texcoords) m.UV.assign(d.texcoords, d.texcoords + 2 * d.num_vertices);
        m.F.assign(d.indices, d.indices + 3 * d.num_triangles);
        m.material = d.material;
        m.light = -1;
        m.prim_offset = off;
        off += d.num_triangles;
        if (d.material < 0 || d.material >= nmat) {
            g_error = "mesh material out of range";
            delete sc;
            return nullptr;
        }
        // mesh.cpp:21-28
        for (uint32_t f = 0; f < m.tri_count(); f++) m.dpdf.append(m.area(f));
        m.dpdf.normalize();
        sc->meshes.push_back(std::move(m));
    }
    for (int l = 0; l < nl; l++) {
        Light L;
        L.type = lights[l].type;
        L.mesh = lights[l].mesh;
        L.radiance = ld3(lights[l].radiance);
        L.position = ld3(lights[l].position);
        if (L.type == DL_LIGHT_AREA) {
            if (L.mesh < 0 || L.mesh >= nm) {
                g_error = "area light mesh out of range";
                delete sc;
                return nullptr;
            }
            sc->meshes[L.mesh].light = l;
        } else if (L.type == DL_LIGHT_ENVMAP) {
            const dl_light_desc& d = lights[l];
            if (sc->env_light >= 0 || !d.env_rgb || d.env_width <= 0 || d.env_height <= 0) {
                g_error = "bad envmap (at most one, with texels)";
                delete sc;
                return nullptr;
            }
            L.env_w = d.env_width;
            L.env_h = d.env_height;
            L.env_scale = d.env_scale;
            L.env_visual = d.env_visual != 0;
            L.env_bg = ld3(d.env_background);
            L.env_rgb.assign(d.env_rgb, d.env_rgb + 3 * (size_t)d.env_width * d.env_height);
            env_build(L);
            sc->env_light = l;
        } else if (L.type != DL_LIGHT_POINT) {
            g_error = "bad light type";
            delete sc;
            return nullptr;
        }
        sc->lights.push_back(L);
    }
    // Power-proportional emitter pick, as the renderer defines it (no
    // reference counterpart): area pi*A*max(L), point 4pi*max(I), envmap
    // pi*R^2*integral*|scale| with R half the diagonal of the box of all
    // vertices; alias table in double over these weights.
    {
        const double kPiD = 3.14159265358979323846;
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        bool any = false;
        for (const Mesh& m : sc->meshes)
            for (size_t k = 0; k < m.V.size(); k++) {
                lo[k % 3] = std::min(lo[k % 3], (double)m.V[k]);
                hi[k % 3] = std::max(hi[k % 3], (double)m.V[k]);
                any = true;
            }
        double r2 = 0.0;
        if (any)
            for (int k = 0; k < 3; k++) r2 += 0.25 * (hi[k] - lo[k]) * (hi[k] - lo[k]);
        const size_t N = sc->lights.size();
        std::vector<double> w(N, 0.0), q(N, 1.0);
        sc->pick_alias.resize(N);
        for (size_t l = 0; l < N; l++) {
            const Light& L = sc->lights[l];
            double m = std::max(L.radiance.x, std::max(L.radiance.y, L.radiance.z));
            if (L.type == DL_LIGHT_AREA) {
                double area = 0.0;
                const Mesh& me = sc->meshes[L.mesh];
                for (uint32_t f = 0; f < me.tri_count(); f++) area += (double)me.area(f);
                w[l] = kPiD * area * std::max(m, 0.0);
            } else if (L.type == DL_LIGHT_POINT) {
                w[l] = 4.0 * kPiD * std::max(m, 0.0);
            } else {
                w[l] = kPiD * r2 * L.env_sum * (double)std::fabs(L.env_scale);
            }
        }
        double sum = 0.0;
        for (size_t l = 0; l < N; l++) sum += w[l];
        for (size_t l = 0; l < N; l++) sc->pick_alias[l] = (uint32_t)l;
        if (sum > 0.0) {
            for (size_t l = 0; l < N; l++) q[l] = (double)N * w[l] / sum;
            std::vector<uint32_t> part(N);
            uint32_t s = 0u, large = (uint32_t)N;
            for (uint32_t l = 0; l < N; l++) part[(q[l] < 1.0) ? (s++) : (--large)] = l;
            for (s = 0; s < large && large < N; ++s) {
                const uint32_t j = part[s], k = part[large];
                sc->pick_alias[j] = k;
                q[k] += q[j] - 1.0;
                large = (q[k] < 1.0) ? (large + 1u) : large;
            }
        }
        sc->pick_q.resize(N);
        sc->pick_prob.resize(N);
        for (size_t l = 0; l < N; l++) {
            sc->pick_q[l] = (float)q[l];
            sc->pick_prob[l] = sum > 0.0 ? (float)(w[l] / sum) : 1.0f / (float)N;
        }
    }
    // OCTree::build (octree.cpp:135-151): meshes in scene order.
    BBox box;
    std::vector<std::pair<int, int>> tris;
    for (int i = 0; i < nm; i++) {
        for (uint32_t j = 0; j < sc->meshes[i].tri_count(); j++) tris.push_back({i, (int)j});
        BBox mb;
        const Mesh& m = sc->meshes[i];
        for (size_t k = 0; k + 2 < m.V.size(); k += 3) mb.expand(V3(m.V[k], m.V[k + 1], m.V[k + 2]));
        box.expand(mb);
    }
    sc->root = build_node(*sc, box, tris);
    sc->cam = make_camera(*cam);
    sc->filter = make_filter(filter);
    return sc;
}

void orc_scene_destroy(void* p) { delete static_cast<Scene*>(p); }

int orc_trace_closest(void* p, const float* rays, int64_t n, int32_t* prim, float* t, float* u,
                      float* v, int32_t threads) {
    const Scene& sc = *static_cast<Scene*>(p);
    parallel(threads, n, [&](int, int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) {
            const float* r = rays + 8 * i;
            Ray ray = make_ray(V3(r[0], r[1], r[2]), V3(r[4], r[5], r[6]), r[3], r[7]);
            P2 uv{0, 0};
            float tt = 0;
            std::pair<int, int> f(-1, -1);
            if (closest(sc, sc.root, ray, uv, tt, f)) {
                prim[i] = (int32_t)(sc.meshes[f.first].prim_offset + f.second);
                t[i] = tt;
                u[i] = uv.x;
                v[i] = uv.y;
            } else {
                prim[i] = -1;
                t[i] = u[i] = v[i] = 0.f;
            }
        }
    });
    return 0;
}

int orc_trace_any(void* p, const float* rays, int64_t n, uint8_t* occ, int32_t threads) {
    const Scene& sc = *static_cast<Scene*>(p);
    parallel(threads, n, [&](int, int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) {
            const float* r = rays + 8 * i;
            Ray ray = make_ray(V3(r[0], r[1], r[2]), V3(r[4], r[5], r[6]), r[3], r[7]);
            occ[i] = occluded(sc, ray) ? 1 : 0;
        }
    });
    return 0;
}

// The block renderer over the listed blocks of the spiral order (all of
// them when `list` is null), each block with its own pcg32 seeded from the
// block offset as Independent::prepare does.
static int render_block_list(const Scene& sc, const dl_render_opts* opts, int32_t threads,
                             const std::vector<std::pair<int, int>>& blocks, float* rgb_out, float* film_out,
                             double* seconds) {
    Opts o = opts_of(opts);
    int spp = opts ? opts->spp : 1;
    const int BS = 32;
    Film film;
    film.reset(0, 0, sc.cam.w, sc.cam.h, sc.filter.border);
    std::mutex mu;
    std::atomic<size_t> next(0);
    auto t0 = std::chrono::steady_clock::now();
    parallel(threads, threads, [&](int, int64_t, int64_t) {
        Film blk;
        Pcg32 rng;
        while (true) {
            size_t k = next.fetch_add(1);
            if (k >= blocks.size()) break;
            int bx = blocks[k].first, by = blocks[k].second;
            int bw = std::min(BS, sc.cam.w - bx), bh = std::min(BS, sc.cam.h - by);
            blk.reset(bx, by, bw, bh, sc.filter.border);
            rng.seed((uint64_t)bx, (uint64_t)by);  // independent.cpp:30-35
            for (int y = 0; y < bh; ++y)
                for (int x = 0; x < bw; ++x)
                    for (int i = 0; i < spp; ++i) {
                        P2 ps = rng.next2d();
                        ps = P2{(float)(x + bx) + ps.x, (float)(y + by) + ps.y};
                        (void)rng.next2d();  // aperture sample, unused by "virtual"
                        Ray ray = camera_ray(sc.cam, ps);
                        V3 val = Li(sc, rng, ray, o);
                        film_put(blk, sc.filter, ps, val);
                    }
            std::lock_guard<std::mutex> lk(mu);
            film_merge(film, blk);
        }
    });
    auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    film_outputs(film, rgb_out, film_out);
    return 0;
}

int orc_render_blocks(void* p, const dl_render_opts* opts, int32_t threads, int32_t max_blocks,
                      float* rgb_out, float* film_out, double* seconds) {
    const Scene& sc = *static_cast<Scene*>(p);
    auto blocks = spiral_blocks(sc.cam.w, sc.cam.h, 32);
    if (max_blocks > 0 && (size_t)max_blocks < blocks.size()) blocks.resize(max_blocks);
    return render_block_list(sc, opts, threads, blocks, rgb_out, film_out, seconds);
}

int orc_render_block_subset(void* p, const dl_render_opts* opts, int32_t threads, int32_t n,
                            const int32_t* spiral_index, float* rgb_out, float* film_out, double* seconds) {
    const Scene& sc = *static_cast<Scene*>(p);
    auto all = spiral_blocks(sc.cam.w, sc.cam.h, 32);
    std::vector<std::pair<int, int>> blocks;
    for (int32_t i = 0; i < n; i++) {
        if (spiral_index[i] < 0 || (size_t)spiral_index[i] >= all.size()) return 1;
        blocks.push_back(all[spiral_index[i]]);
    }
    return render_block_list(sc, opts, threads, blocks, rgb_out, film_out, seconds);
}

int orc_num_blocks(void* p) {
    const Scene& sc = *static_cast<Scene*>(p);
    return (int)spiral_blocks(sc.cam.w, sc.cam.h, 32).size();
}

int orc_li(void* p, const dl_render_opts* opts, int64_t n, const int32_t* xys, float* L,
           float* pos, int32_t threads) {
    const Scene& sc = *static_cast<Scene*>(p);
    Opts o = opts_of(opts);
    uint64_t seed = opts ? opts->seed : 0;
    parallel(threads, n, [&](int, int64_t b, int64_t e) {
        Pcg32 rng;
        for (int64_t i = b; i < e; i++) {
            int x = xys[3 * i], y = xys[3 * i + 1], s = xys[3 * i + 2];
            seed_path(rng, seed, sc.cam.w, sc.cam.h, x, y, s);
            P2 ps = rng.next2d();
            ps = P2{(float)x + ps.x, (float)y + ps.y};
            (void)rng.next2d();
            V3 val = Li(sc, rng, camera_ray(sc.cam, ps), o);
            L[3 * i] = val.x; L[3 * i + 1] = val.y; L[3 * i + 2] = val.z;
            if (pos) { pos[2 * i] = ps.x; pos[2 * i + 1] = ps.y; }
        }
    });
    return 0;
}

int orc_render_paths(void* p, const dl_render_opts* opts, int32_t threads, float* rgb_out,
                     float* film_out, double* seconds) {
    const Scene& sc = *static_cast<Scene*>(p);
    Opts o = opts_of(opts);
    int spp = opts ? opts->spp : 1;
    int s0 = opts ? opts->spp_offset : 0;
    uint64_t seed = opts ? opts->seed : 0;
    int T = std::max(1, threads);
    std::vector<Film> films(T);
    auto t0 = std::chrono::steady_clock::now();
    parallel(T, (int64_t)sc.cam.h, [&](int k, int64_t b, int64_t e) {
        Film& f = films[k];
        f.reset(0, 0, sc.cam.w, sc.cam.h, sc.filter.border);
        Pcg32 rng;
        for (int64_t y = b; y < e; y++)
            for (int x = 0; x < sc.cam.w; x++)
                for (int s = s0; s < s0 + spp; s++) {
                    seed_path(rng, seed, sc.cam.w, sc.cam.h, x, (int)y, s);
                    P2 ps = rng.next2d();
                    ps = P2{(float)x + ps.x, (float)y + ps.y};
                    (void)rng.next2d();
                    V3 val = Li(sc, rng, camera_ray(sc.cam, ps), o);
                    film_put(f, sc.filter, ps, val);
                }
    });
    for (int k = 1; k < T; k++)
        for (size_t i = 0; i < films[0].px.size(); i++) films[0].px[i] += films[k].px[i];
    auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    film_outputs(films[0], rgb_out, film_out);
    return 0;
}

int orc_bsdf_query(const dl_material_desc* md, int64_t n, const float* wi, const float* wo,
                   const float* smp, float* eval, float* pdf, float* s_wo, float* s_w,
                   float* s_eta, int32_t* s_measure) {
    Material m;
    m.type = md->type;
    m.albedo = ld3(md->albedo);
    m.specular = ld3(md->specular);
    m.ax = md->alpha[0];
    m.ay = md->alpha[1];
    m.int_ior = md->int_ior;
    m.ext_ior = md->ext_ior;
    m.ks = 1 - maxc(m.albedo);
    for (int64_t i = 0; i < n; i++) {
        BRec q;
        q.wi = ld3(wi + 3 * i);
        q.wo = ld3(wo + 3 * i);
        q.measure = kSolidAngle;
        V3 e = bsdf_eval(m, q);
        eval[3 * i] = e.x; eval[3 * i + 1] = e.y; eval[3 * i + 2] = e.z;
        pdf[i] = bsdf_pdf(m, q);
        BRec s;
        s.wi = ld3(wi + 3 * i);
        V3 w = bsdf_sample(m, s, P2{smp[3 * i], smp[3 * i + 1]}, smp[3 * i + 2]);
        s_wo[3 * i] = s.wo.x; s_wo[3 * i + 1] = s.wo.y; s_wo[3 * i + 2] = s.wo.z;
        s_w[3 * i] = w.x; s_w[3 * i + 1] = w.y; s_w[3 * i + 2] = w.z;
        s_eta[i] = s.eta;
        s_measure[i] = s.measure;
    }
    return 0;
}

int orc_frame(int64_t n, const float* nrm, float* t, float* b) {
    for (int64_t i = 0; i < n; i++) {
        Frame f = make_frame(ld3(nrm + 3 * i));
        t[3 * i] = f.t.x; t[3 * i + 1] = f.t.y; t[3 * i + 2] = f.t.z;
        b[3 * i] = f.b.x; b[3 * i + 1] = f.b.y; b[3 * i + 2] = f.b.z;
    }
    return 0;
}

int orc_emitter_sample(void* p, const dl_render_opts* opts, int64_t n, const float* pts,
                       const float* nrm, const float* smp, float* d, float* dist, float* pdf,
                       float* spec) {
    const Scene& sc = *static_cast<Scene*>(p);
    uint32_t flags = opts ? opts->flags : 0;
    for (int64_t i = 0; i < n; i++) {
        Hit its;
        its.p = ld3(pts + 3 * i);
        its.sh = make_frame(ld3(nrm + 3 * i));
        its.geo = its.sh;
        DirSample ds;
        V3 sp;
        bool delta;
        sample_emitter(sc, its, P2{smp[2 * i], smp[2 * i + 1]}, ds, sp, delta, flags, nullptr);
        d[3 * i] = ds.d.x; d[3 * i + 1] = ds.d.y; d[3 * i + 2] = ds.d.z;
        spec[3 * i] = sp.x; spec[3 * i + 1] = sp.y; spec[3 * i + 2] = sp.z;
        dist[i] = ds.dist;
        pdf[i] = ds.pdf;
    }
    return 0;
}

int orc_env_tables(void* p, float* q, uint32_t* alias, float* pdf) {
    const Scene& sc = *static_cast<Scene*>(p);
    if (sc.env_light < 0) return 1;
    const Light& L = sc.lights[sc.env_light];
    size_t n = (size_t)L.env_w * L.env_h;
    std::copy(L.env_q.begin(), L.env_q.begin() + n, q);
    std::copy(L.env_alias.begin(), L.env_alias.begin() + n, alias);
    std::copy(L.env_pdf.begin(), L.env_pdf.begin() + n, pdf);
    return 0;
}

int orc_env_query(void* p, int64_t n, const float* xi, const float* nrm, const float* dirs, float* s_dir,
                  float* s_pdf, float* s_val, float* pdf, float* val) {
    const Scene& sc = *static_cast<Scene*>(p);
    if (sc.env_light < 0) return 1;
    const Light& L = sc.lights[sc.env_light];
    for (int64_t i = 0; i < n; i++) {
        Hit its;
        its.sh = make_frame(ld3(nrm + 3 * i));
        DirSample ds;
        V3 r = env_sample(L, its, ld3(xi + 3 * i), ds);
        s_dir[3 * i] = ds.d.x; s_dir[3 * i + 1] = ds.d.y; s_dir[3 * i + 2] = ds.d.z;
        s_pdf[i] = ds.pdf;
        s_val[3 * i] = r.x; s_val[3 * i + 1] = r.y; s_val[3 * i + 2] = r.z;
        V3 d = ld3(dirs + 3 * i);
        pdf[i] = env_pdf(L, d);
        V3 v = env_eval(L, d);
        val[3 * i] = v.x; val[3 * i + 1] = v.y; val[3 * i + 2] = v.z;
    }
    return 0;
}

int orc_env_miss(void* p, const dl_render_opts* opts, int64_t n, const float* dirs, const int32_t* depth,
                 const float* bsdf_pdf, const uint8_t* is_diffuse, float* out) {
    const Scene& sc = *static_cast<Scene*>(p);
    if (sc.env_light < 0) return 1;
    uint32_t flags = opts ? opts->flags : 0;
    for (int64_t i = 0; i < n; i++) {
        float w;
        V3 le = env_miss(sc, ld3(dirs + 3 * i), depth[i] == 0, is_diffuse[i] != 0, bsdf_pdf[i], flags, w);
        out[3 * i] = w * le.x; out[3 * i + 1] = w * le.y; out[3 * i + 2] = w * le.z;
    }
    return 0;
}

int orc_camera_ray(void* p, int64_t n, const float* film, float* o, float* d) {
    const Scene& sc = *static_cast<Scene*>(p);
    for (int64_t i = 0; i < n; i++) {
        Ray r = camera_ray(sc.cam, P2{film[2 * i], film[2 * i + 1]});
        o[3 * i] = r.o.x; o[3 * i + 1] = r.o.y; o[3 * i + 2] = r.o.z;
        d[3 * i] = r.d.x; d[3 * i + 1] = r.d.y; d[3 * i + 2] = r.d.z;
    }
    return 0;
}

int orc_hit_data(void* p, int64_t n, const int32_t* prim, const float* bary, float* sn, float* gn, float* st,
                 float* tuv) {
    const Scene& sc = *static_cast<Scene*>(p);
    for (int64_t i = 0; i < n; i++) {
        int mi = -1;
        for (size_t k = 0; k < sc.meshes.size(); k++)
            if (prim[i] >= sc.meshes[k].prim_offset &&
                prim[i] < sc.meshes[k].prim_offset + (int64_t)sc.meshes[k].tri_count())
                mi = (int)k;
        if (mi < 0) return 1;
        Hit its;
        fill_hit(sc, mi, (int)(prim[i] - sc.meshes[mi].prim_offset), P2{bary[2 * i], bary[2 * i + 1]}, 1.f, its);
        sn[3 * i] = its.sh.n.x; sn[3 * i + 1] = its.sh.n.y; sn[3 * i + 2] = its.sh.n.z;
        gn[3 * i] = its.geo.n.x; gn[3 * i + 1] = its.geo.n.y; gn[3 * i + 2] = its.geo.n.z;
        st[3 * i] = its.tan.x; st[3 * i + 1] = its.tan.y; st[3 * i + 2] = its.tan.z;
        tuv[2 * i] = its.tuv.x; tuv[2 * i + 1] = its.tuv.y;
    }
    return 0;
}

int orc_pcg32(uint64_t initstate, uint64_t initseq, int32_t n, uint32_t* out, float* out_float) {
    Pcg32 a, b;
    a.seed(initstate, initseq);
    b.seed(initstate, initseq);
    for (int32_t i = 0; i < n; i++) {
        out[i] = a.next_u32();
        out_float[i] = b.next_float();
    }
    return 0;
}

}  // extern "C"
