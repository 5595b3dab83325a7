// Device code shared by the trace and render kernels (sm_103a).
//
// The shading math restates the reference CPU path (paths relative to the
// reference project root; the same steps as the CPU oracle):
//   Moller-Trumbore        src/tracer/mesh/mesh.cpp:180-220 (bit-exact: _rn
//                          intrinsics, no contraction, IEEE division)
//   shading frame          include/core/math/frame.h:104-123, octree.cpp:193-209
//   warps                  src/core/math/wrap.cpp:33-97
//   BSDFs                  src/tracer/bsdf/{diffuse,mirror,dielectric,microfacet}.cpp,
//                          src/optix/cuda/material/aniso_ggx.cu
//   emitters               src/tracer/emitter/{area,point}.cpp, scene.cpp:139-179
//   camera                 src/tracer/camera/virtual.cpp:52-65
//   film splat             src/core/bitmap/block.cpp:81-113
// Transcendentals use CUDA's single-precision functions where the reference
// evaluates libm in double; results then agree to a few ulps.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/drawlab.h"
#include "layout.h"

namespace dl {

// ------------------------------------------------------------ float3 math
__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 add(float3 a, float3 b) { return f3(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)); }
__device__ __forceinline__ float3 sub(float3 a, float3 b) { return f3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)); }
__device__ __forceinline__ float3 neg(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 scale(float3 a, float s) { return f3(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)); }
__device__ __forceinline__ float3 divs(float3 a, float s) { return f3(__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s)); }
__device__ __forceinline__ float3 mul(float3 a, float3 b) { return f3(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)); }
__device__ __forceinline__ float dot(float3 a, float3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return f3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
              __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
              __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float length(float3 a) { return __fsqrt_rn(dot(a, a)); }
__device__ __forceinline__ float3 normalize(float3 a) {
    float l = length(a);
    return f3(__fdiv_rn(a.x, l), __fdiv_rn(a.y, l), __fdiv_rn(a.z, l));
}
__device__ __forceinline__ float maxc(float3 a) { return fmaxf(fmaxf(a.x, a.y), a.z); }
__device__ __forceinline__ float3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }
__device__ __forceinline__ float3 xyz(float4 a) { return f3(a.x, a.y, a.z); }

// ------------------------------------------------------------------ pcg32
// PCG32 (O'Neill 2014, XSH-RR) with the seeding and float construction of the
// pcg32 header the reference sampler uses (src/tracer/sampler/independent.cpp).
struct Pcg32 {
    uint64_t state, inc;
    __device__ __forceinline__ uint32_t next_u32() {
        uint64_t old = state;
        state = old * 0x5851f42d4c957f2dULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((~rot + 1u) & 31));
    }
    __device__ __forceinline__ void seed(uint64_t initstate, uint64_t initseq) {
        state = 0u;
        inc = (initseq << 1u) | 1u;
        next_u32();
        state += initstate;
        next_u32();
    }
    __device__ __forceinline__ float next_float() {
        return __uint_as_float((next_u32() >> 9) | 0x3f800000u) - 1.0f;
    }
    // Independent::next2D as compiled for the reference: the first draw is y.
    __device__ __forceinline__ float2 next2d() {
        float first = next_float();
        float second = next_float();
        return make_float2(second, first);
    }
};

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// Stream of path (x, y, s): initseq = s*W*H + y*W + x,
// initstate = splitmix64(initseq ^ splitmix64(seed)).
__device__ __forceinline__ void seed_path(Pcg32& r, uint64_t seed_mix, int w, int h, int x, int y, int s) {
    uint64_t seq = (uint64_t)s * (uint64_t)w * (uint64_t)h + (uint64_t)y * (uint64_t)w + (uint64_t)x;
    r.seed(splitmix64(seq ^ seed_mix), seq);
}

// ---------------------------------------------------------- intersection
// Moller-Trumbore exactly as mesh.cpp:180-220.
__device__ __forceinline__ bool intersect_tri(float3 v0, float3 v1, float3 v2, float3 o, float3 d,
                                              float tmin, float tmax, float& t, float& u, float& v) {
    float3 e1 = sub(v1, v0), e2 = sub(v2, v0);
    float3 pvec = cross(d, e2);
    float det = dot(e1, pvec);
    if (det > -1e-8f && det < 1e-8f) return false;
    float inv = __fdiv_rn(1.0f, det);
    float3 tvec = sub(o, v0);
    u = __fmul_rn(dot(tvec, pvec), inv);
    if (u < 0.0f || u > 1.0f) return false;
    float3 qvec = cross(tvec, e1);
    v = __fmul_rn(dot(d, qvec), inv);
    if (v < 0.0f || __fadd_rn(u, v) > 1.0f) return false;
    t = __fmul_rn(dot(e2, qvec), inv);
    return t >= tmin && t <= tmax;
}

struct RayBox {
    float3 idir, ood;
};
__device__ __forceinline__ float safe_rcp(float x) {
    return 1.0f / (fabsf(x) > 1e-20f ? x : copysignf(1e-20f, x));
}
__device__ __forceinline__ RayBox make_raybox(float3 o, float3 d) {
    RayBox r;
    r.idir = f3(safe_rcp(d.x), safe_rcp(d.y), safe_rcp(d.z));
    r.ood = f3(o.x * r.idir.x, o.y * r.idir.y, o.z * r.idir.z);
    return r;
}
// Slab test of both children of a node; the far distance is widened by
// 1 + 2*gamma(3) so the float test is conservative (boxes are also padded).
__device__ __forceinline__ void box2(const RayBox& rb, float tmin, float tmax, float4 a, float4 b,
                                     float4 c, bool& h0, bool& h1, float& t0, float& t1) {
    const float grow = 1.0000004f;
    float x0 = fmaf(a.x, rb.idir.x, -rb.ood.x), x1 = fmaf(a.y, rb.idir.x, -rb.ood.x);
    float y0 = fmaf(a.z, rb.idir.y, -rb.ood.y), y1 = fmaf(a.w, rb.idir.y, -rb.ood.y);
    float z0 = fmaf(c.x, rb.idir.z, -rb.ood.z), z1 = fmaf(c.y, rb.idir.z, -rb.ood.z);
    float n0 = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), tmin));
    float f0 = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), tmax)) * grow;
    float X0 = fmaf(b.x, rb.idir.x, -rb.ood.x), X1 = fmaf(b.y, rb.idir.x, -rb.ood.x);
    float Y0 = fmaf(b.z, rb.idir.y, -rb.ood.y), Y1 = fmaf(b.w, rb.idir.y, -rb.ood.y);
    float Z0 = fmaf(c.z, rb.idir.z, -rb.ood.z), Z1 = fmaf(c.w, rb.idir.z, -rb.ood.z);
    float n1 = fmaxf(fmaxf(fminf(X0, X1), fminf(Y0, Y1)), fmaxf(fminf(Z0, Z1), tmin));
    float f1 = fminf(fminf(fmaxf(X0, X1), fmaxf(Y0, Y1)), fminf(fmaxf(Z0, Z1), tmax)) * grow;
    h0 = n0 <= f0;
    h1 = n1 <= f1;
    t0 = n0;
    t1 = n1;
}

struct TraversalCounters {
    unsigned long long nodes;
    unsigned long long tris;
};

// Closest hit over the BVH.  Returns the leaf-order triangle index or -1;
// t/u/v as the reference's Moller-Trumbore computes them.  `err` is set when
// the stack would overflow (cannot happen for depth <= kStackSize builds).
template <bool kCount>
__device__ __forceinline__ int trace_closest(const DevScene& sc, float3 o, float3 d, float tmin,
                                             float tmax, float& ht, float& hu, float& hv,
                                             uint32_t& err, uint32_t& n_nodes, uint32_t& n_tris) {
    int hit = -1;
    if (sc.num_tris == 0) return -1;
    RayBox rb = make_raybox(o, d);
    int stack[kStackSize];
    int sp = 0;
    int node = 0;
    for (;;) {
        if (node >= 0) {
#ifdef DL_CHECKS
            if (node >= sc.num_nodes) {  // bounds-checked build: bit 4 of the error word
                err |= 4u;
                break;
            }
#endif
            const float4* np = sc.nodes + 4 * node;
            float4 a = __ldg(np), b = __ldg(np + 1), c = __ldg(np + 2);
            int4 ch = __ldg(reinterpret_cast<const int4*>(np + 3));
            if (kCount) n_nodes++;
            bool h0, h1;
            float t0, t1;
            box2(rb, tmin, tmax, a, b, c, h0, h1, t0, t1);
            h0 = h0 && ch.x != kEmptyChild;
            h1 = h1 && ch.y != kEmptyChild;
            if (h0 && h1) {
                int near = ch.x, far = ch.y;
                if (t1 < t0) { near = ch.y; far = ch.x; }
                if (sp < kStackSize) stack[sp++] = far; else err |= 1u;
                node = near;
                continue;
            } else if (h0) {
                node = ch.x;
                continue;
            } else if (h1) {
                node = ch.y;
                continue;
            }
        } else {
            int ref = ~node;
            int first = ref >> 4, count = (ref & 15) + 1;
#ifdef DL_CHECKS
            if (first < 0 || first + count > sc.num_tris) {
                err |= 4u;
                count = 0;
            }
#endif
            for (int k = 0; k < count; k++) {
                const float4* tp = sc.tris + 3 * (first + k);
                float4 p0 = __ldg(tp), p1 = __ldg(tp + 1), p2 = __ldg(tp + 2);
                if (kCount) n_tris++;
                float t, u, v;
                if (intersect_tri(xyz(p0), xyz(p1), xyz(p2), o, d, tmin, tmax, t, u, v)) {
                    tmax = t;
                    ht = t;
                    hu = u;
                    hv = v;
                    hit = first + k;
                }
            }
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
    return hit;
}

// Any hit (shadow rays), first accepted triangle ends the query.
template <bool kCount>
__device__ __forceinline__ bool trace_any(const DevScene& sc, float3 o, float3 d, float tmin,
                                          float tmax, uint32_t& err, uint32_t& n_nodes,
                                          uint32_t& n_tris) {
    if (sc.num_tris == 0) return false;
    RayBox rb = make_raybox(o, d);
    int stack[kStackSize];
    int sp = 0;
    int node = 0;
    for (;;) {
        if (node >= 0) {
#ifdef DL_CHECKS
            if (node >= sc.num_nodes) {  // bounds-checked build: bit 4 of the error word
                err |= 4u;
                break;
            }
#endif
            const float4* np = sc.nodes + 4 * node;
            float4 a = __ldg(np), b = __ldg(np + 1), c = __ldg(np + 2);
            int4 ch = __ldg(reinterpret_cast<const int4*>(np + 3));
            if (kCount) n_nodes++;
            bool h0, h1;
            float t0, t1;
            box2(rb, tmin, tmax, a, b, c, h0, h1, t0, t1);
            h0 = h0 && ch.x != kEmptyChild;
            h1 = h1 && ch.y != kEmptyChild;
            if (h0 && h1) {
                int near = ch.x, far = ch.y;
                if (t1 < t0) { near = ch.y; far = ch.x; }
                if (sp < kStackSize) stack[sp++] = far; else err |= 1u;
                node = near;
                continue;
            } else if (h0) {
                node = ch.x;
                continue;
            } else if (h1) {
                node = ch.y;
                continue;
            }
        } else {
            int ref = ~node;
            int first = ref >> 4, count = (ref & 15) + 1;
#ifdef DL_CHECKS
            if (first < 0 || first + count > sc.num_tris) {
                err |= 4u;
                count = 0;
            }
#endif
            for (int k = 0; k < count; k++) {
                const float4* tp = sc.tris + 3 * (first + k);
                float4 p0 = __ldg(tp), p1 = __ldg(tp + 1), p2 = __ldg(tp + 2);
                if (kCount) n_tris++;
                float t, u, v;
                if (intersect_tri(xyz(p0), xyz(p1), xyz(p2), o, d, tmin, tmax, t, u, v)) return true;
            }
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
    return false;
}

// ------------------------------------------------------------------ frames
struct Frame {
    float3 t, b, n;
};
// frame.h:113-123 (n is not normalised by the reference's constructor)
__device__ __forceinline__ Frame make_frame(float3 n) {
    Frame f;
    f.n = n;
    float3 t;
    if (fabsf(__fsub_rn(n.z, 1.0f)) > kRayEps && fabsf(__fadd_rn(n.z, 1.0f)) > kRayEps)
        t = f3(0.f, 0.f, 1.f);
    else
        t = f3(1.f, 0.f, 0.f);
    f.b = normalize(cross(n, t));
    f.t = cross(f.b, n);
    return f;
}
// Onb(normal, 0) of include/optix/math/onb.h:11-33 (frame of aniso_ggx)
__device__ __forceinline__ Frame make_onb(float3 n) {
    Frame f;
    f.n = n;
    float3 bn = fabsf(n.x) > fabsf(n.z) ? f3(-n.y, n.x, 0.f) : f3(0.f, -n.z, n.y);
    f.b = normalize(bn);
    f.t = cross(f.b, n);
    return f;
}
// Onb(normal, tangent) with a given (non-zero) tangent (onb.h:29-32): the
// tangent as given, binormal = normalize(n x t).
__device__ __forceinline__ Frame make_onb_t(float3 n, float3 t) {
    if (t.x == 0.f && t.y == 0.f && t.z == 0.f) return make_onb(n);
    Frame f;
    f.n = n;
    f.t = t;
    f.b = normalize(cross(n, t));
    return f;
}
__device__ __forceinline__ float3 to_local(const Frame& f, float3 v) {
    return f3(dot(v, f.t), dot(v, f.b), dot(f.n, v));
}
__device__ __forceinline__ float3 to_world(const Frame& f, float3 v) {
    return add(add(scale(f.t, v.x), scale(f.b, v.y)), scale(f.n, v.z));
}

// ------------------------------------------------------------------ warps
__device__ __forceinline__ float2 square_to_uniform_disk(float2 s) {
    float r = __fsqrt_rn(s.x);
    float theta = __fmul_rn(__fmul_rn(2.0f, kPiF), s.y);
    float sn, cs;
    sincosf(theta, &sn, &cs);
    return make_float2(__fmul_rn(r, cs), __fmul_rn(r, sn));
}
__device__ __forceinline__ float3 square_to_cosine_hemisphere(float2 s) {
    float2 p = square_to_uniform_disk(s);
    float sum = __fadd_rn(__fmul_rn(p.x, p.x), __fmul_rn(p.y, p.y));
    return f3(p.x, p.y, __fsqrt_rn(__fsub_rn(1.0f, sum)));
}
__device__ __forceinline__ float cosine_hemisphere_pdf(float3 v) { return v.z <= 0.f ? 0.f : __fmul_rn(v.z, kInvPiF); }
__device__ __forceinline__ float3 square_to_beckmann(float2 s, float alpha) {
    float theta = atanf(__fsqrt_rn(__fmul_rn(__fmul_rn(-alpha, alpha), logf(__fsub_rn(1.0f, s.x)))));
    float phi = __fmul_rn(__fmul_rn(2.0f, kPiF), s.y);
    float st, ct, sp, cp;
    sincosf(theta, &st, &ct);
    sincosf(phi, &sp, &cp);
    return f3(__fmul_rn(st, cp), __fmul_rn(st, sp), ct);
}
__device__ __forceinline__ float beckmann_pdf(float3 m, float alpha) {
    if (m.z <= 0.f) return 0.f;
    float c = m.z;
    float cc = __fmul_rn(c, c);
    float tan2 = __fdiv_rn(__fsub_rn(1.0f, cc), cc);
    float e = expf(__fdiv_rn(-tan2, __fmul_rn(alpha, alpha)));
    float den = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(alpha, alpha), c), c), c);
    return __fdiv_rn(__fmul_rn(kInvTwoPiF, __fmul_rn(2.0f, e)), den);
}
__device__ __forceinline__ float3 square_to_uniform_triangle(float2 s) {
    float t = __fsqrt_rn(__fsub_rn(1.f, s.x));
    float ty = __fmul_rn(t, s.y);
    return f3(__fsub_rn(1.f, t), ty, __fsub_rn(t, ty));
}

__device__ __forceinline__ float fresnel(float cosI, float extIOR, float intIOR) {
    float etaI = extIOR, etaT = intIOR;
    if (extIOR == intIOR) return 0.0f;
    if (cosI < 0.0f) {
        float tmp = etaI; etaI = etaT; etaT = tmp;
        cosI = -cosI;
    }
    float eta = __fdiv_rn(etaI, etaT);
    float sinT2 = __fmul_rn(__fmul_rn(eta, eta), __fsub_rn(1.f, __fmul_rn(cosI, cosI)));
    if (sinT2 > 1.0f) return 1.0f;
    float cosT = __fsqrt_rn(__fsub_rn(1.0f, sinT2));
    float a = __fmul_rn(etaI, cosI), b = __fmul_rn(etaT, cosT);
    float Rs = __fdiv_rn(__fsub_rn(a, b), __fadd_rn(a, b));
    float c = __fmul_rn(etaT, cosI), e = __fmul_rn(etaI, cosT);
    float Rp = __fdiv_rn(__fsub_rn(c, e), __fadd_rn(c, e));
    return __fdiv_rn(__fadd_rn(__fmul_rn(Rs, Rs), __fmul_rn(Rp, Rp)), 2.0f);
}
__device__ __forceinline__ float3 refract(float3 wi, float eta) {
    float cosI = wi.z;
    bool outside = cosI > 0.f;
    eta = outside ? eta : __fdiv_rn(1.f, eta);
    float cosT2 = __fsub_rn(1.f, __fmul_rn(__fmul_rn(eta, eta), __fsub_rn(1.f, __fmul_rn(cosI, cosI))));
    float cosT = __fsqrt_rn(cosT2);
    cosT = outside ? -cosT : cosT;
    return f3(__fmul_rn(-eta, wi.x), __fmul_rn(-eta, wi.y), cosT);
}
__device__ __forceinline__ float3 reflect(float3 wi, float3 n) {
    return sub(scale(n, __fmul_rn(2.f, dot(wi, n))), wi);
}

// ------------------------------------------------------------------- BSDFs
enum Measure { M_UNKNOWN = 0, M_SOLID = 1, M_DISCRETE = 2 };

struct BRec {
    float3 wi, wo;
    float eta;
    int measure;
};

__device__ __forceinline__ bool is_diffuse(int type) {
    return type == MAT_DIFFUSE || type == MAT_MICROFACET || type == MAT_ANISO_GGX;
}

__device__ __forceinline__ float tan_theta(float3 v) {
    float temp = __fsub_rn(1.f, __fmul_rn(v.z, v.z));
    if (temp <= 0.0f) return 0.0f;
    return __fdiv_rn(__fsqrt_rn(temp), v.z);
}
// microfacet.cpp:35-44 (rational Smith G1), evaluated in float
__device__ __forceinline__ float beckmann_g1(float3 wv, float3 wh, float alpha) {
    float c = __fdiv_rn(dot(wv, wh), wv.z);
    if (c <= 0.f) return 0.f;
    float b = __fdiv_rn(1.0f, __fmul_rn(alpha, tan_theta(wv)));
    if (!(b < 1.6f)) return 1.0f;
    float bb = __fmul_rn(b, b);
    float num = __fadd_rn(__fmul_rn(3.535f, b), __fmul_rn(2.181f, bb));
    float den = __fadd_rn(__fadd_rn(1.f, __fmul_rn(2.276f, b)), __fmul_rn(2.577f, bb));
    return __fdiv_rn(num, den);
}
// aniso_ggx.cu:9-15 and include/optix/math/wrap.h:54-77
__device__ __forceinline__ float ggx_g1(float3 v, float ax, float ay) {
    if (v.z <= 0.f) return 0.f;
    float3 vv = f3(__fmul_rn(v.x, ax), __fmul_rn(v.y, ay), v.z);
    return __fdiv_rn(__fmul_rn(2.0f, v.z), __fadd_rn(v.z, length(vv)));
}
__device__ __forceinline__ float ggx_pdf(float3 m, float ax, float ay) {
    if (m.z <= 0.f) return 0.f;
    float3 h = f3(__fdiv_rn(m.x, ax), __fdiv_rn(m.y, ay), m.z);
    float len2 = dot(h, h);
    return __fdiv_rn(1.f, __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(kPiF, ax), ay), len2), len2));
}
__device__ __forceinline__ float3 square_to_ggx(float2 s, float ax, float ay) {
    float sq = __fdiv_rn(__fsqrt_rn(s.x), __fsqrt_rn(__fsub_rn(1.f, s.x)));
    float sp, cp;
    sincosf(__fmul_rn(__fmul_rn(2.f, kPiF), s.y), &sp, &cp);
    float x = __fmul_rn(__fmul_rn(ax, sq), cp);
    float y = __fmul_rn(__fmul_rn(ay, sq), sp);
    return normalize(f3(-x, -y, 1.f));
}

// BSDF evaluation / density / sampling, specialised per material type T so
// each material kernel carries only its own code.
template <int T>
__device__ __forceinline__ float3 bsdf_eval(const DevMaterial& m, const BRec& r) {
    switch (T) {
        case MAT_DIFFUSE:
            if (r.measure != M_SOLID || r.wi.z <= 0.f || r.wo.z <= 0.f) return f3(0.f, 0.f, 0.f);
            return scale(ld3(m.albedo), kInvPiF);
        case MAT_MICROFACET: {
            float3 wh = normalize(add(r.wi, r.wo));
            float D = beckmann_pdf(wh, m.ax);
            float F = fresnel(dot(r.wi, wh), m.ext_ior, m.int_ior);
            float G = __fmul_rn(beckmann_g1(r.wi, wh, m.ax), beckmann_g1(r.wo, wh, m.ax));
            float deno = __fdiv_rn(1.f, __fmul_rn(__fmul_rn(4.f, r.wi.z), r.wo.z));
            float spec = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(m.ks, D), F), G), deno);
            float3 kd = scale(ld3(m.albedo), kInvPiF);
            return f3(__fadd_rn(kd.x, spec), __fadd_rn(kd.y, spec), __fadd_rn(kd.z, spec));
        }
        case MAT_ANISO_GGX: {
            if (r.wi.z <= 0.f || r.wo.z <= 0.f) return f3(0.f, 0.f, 0.f);
            float3 wh = normalize(add(r.wi, r.wo));
            float D = ggx_pdf(wh, m.ax, m.ay);
            float ldoth = dot(r.wi, wh);
            float temp = fminf(fmaxf(0.0f, __fsub_rn(1.0f, ldoth)), 1.0f);
            float t5 = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(temp, temp), temp), temp), temp);
            float F = __fadd_rn(0.04f, __fmul_rn(0.96f, t5));
            float G = __fmul_rn(ggx_g1(r.wi, m.ax, m.ay), ggx_g1(r.wo, m.ax, m.ay));
            float deno = __fdiv_rn(1.f, __fmul_rn(__fmul_rn(4.f, r.wi.z), r.wo.z));
            float3 spec = scale(scale(scale(scale(ld3(m.specular), D), F), G), deno);
            return add(scale(ld3(m.albedo), kInvPiF), spec);
        }
        default:
            return f3(0.f, 0.f, 0.f);
    }
}

template <int T>
__device__ __forceinline__ float bsdf_pdf(const DevMaterial& m, const BRec& r) {
    switch (T) {
        case MAT_DIFFUSE:
            if (r.measure != M_SOLID || r.wi.z <= 0.f || r.wo.z <= 0.f) return 0.f;
            return __fmul_rn(kInvPiF, r.wo.z);
        case MAT_MICROFACET: {
            if (r.measure != M_SOLID || r.wi.z <= 0.f || r.wo.z <= 0.f) return 0.f;
            float3 wh = normalize(add(r.wi, r.wo));
            float diff = __fmul_rn(__fsub_rn(1.f, m.ks), cosine_hemisphere_pdf(r.wo));
            float spec = __fdiv_rn(__fdiv_rn(__fmul_rn(m.ks, beckmann_pdf(wh, m.ax)), 4.f), dot(wh, r.wo));
            return __fadd_rn(diff, spec);
        }
        case MAT_ANISO_GGX: {
            if (r.measure != M_SOLID || r.wi.z <= 0.f || r.wo.z <= 0.f) return 0.f;
            float3 wh = normalize(add(r.wi, r.wo));
            float diff = __fmul_rn(0.5f, cosine_hemisphere_pdf(r.wo));
            float spec = __fdiv_rn(__fdiv_rn(__fmul_rn(__fmul_rn(0.5f, ggx_pdf(wh, m.ax, m.ay)), wh.z), 4.f),
                                   dot(wh, r.wo));
            return __fadd_rn(diff, spec);
        }
        default:
            return 0.f;
    }
}

// `lobe`: aniso_ggx's third uniform number (aniso_ggx.cu:104-108, drawn
// after the 2D sample; > 0.5 picks the diffuse lobe); unused by the others.
template <int T>
__device__ __forceinline__ float3 bsdf_sample(const DevMaterial& m, BRec& r, float2 s, float lobe) {
    const float3 zero = f3(0.f, 0.f, 0.f);
    switch (T) {
        case MAT_DIFFUSE:
            if (r.wi.z <= 0.f) return zero;
            r.measure = M_SOLID;
            r.wo = square_to_cosine_hemisphere(s);
            r.eta = 1.f;
            return ld3(m.albedo);
        case MAT_MIRROR:
            if (r.wi.z <= 0.f) return zero;
            r.wo = f3(-r.wi.x, -r.wi.y, r.wi.z);
            r.measure = M_DISCRETE;
            r.eta = 1.f;
            return f3(1.f, 1.f, 1.f);
        case MAT_DIELECTRIC: {
            r.measure = M_DISCRETE;
            float cosI = r.wi.z;
            float ri = fresnel(cosI, m.ext_ior, m.int_ior);
            if (s.x < ri) {
                r.wo = f3(-r.wi.x, -r.wi.y, r.wi.z);
                r.eta = 1.f;
            } else {
                float eta = __fdiv_rn(m.ext_ior, m.int_ior);
                r.wo = normalize(refract(r.wi, eta));
                r.eta = cosI > 0.f ? eta : __fdiv_rn(1.f, eta);
            }
            return f3(1.f, 1.f, 1.f);
        }
        case MAT_MICROFACET: {
            if (r.wi.z <= 0.f) return zero;
            r.measure = M_SOLID;
            float sx = s.x;
            float2 ss = s;
            if (sx > m.ks) {
                ss.x = __fdiv_rn(__fsub_rn(sx, m.ks), __fsub_rn(1.f, m.ks));
                r.wo = square_to_cosine_hemisphere(ss);
            } else {
                ss.x = __fdiv_rn(sx, m.ks);
                r.wo = reflect(r.wi, square_to_beckmann(ss, m.ax));
            }
            if (r.wo.z <= 0.f) return zero;
            return divs(scale(bsdf_eval<T>(m, r), r.wo.z), bsdf_pdf<T>(m, r));
        }
        case MAT_ANISO_GGX: {
            if (r.wi.z <= 0.f) return zero;
            r.measure = M_SOLID;
            if (lobe > 0.5f) {
                r.wo = square_to_cosine_hemisphere(s);
            } else {
                r.wo = reflect(r.wi, square_to_ggx(s, m.ax, m.ay));
            }
            if (r.wo.z <= 0.f) return zero;
            return divs(scale(bsdf_eval<T>(m, r), r.wo.z), bsdf_pdf<T>(m, r));
        }
        default:
            return zero;
    }
}

__device__ __forceinline__ float mis_weight(float a, float b) {
    a = __fmul_rn(a, a);
    b = __fmul_rn(b, b);
    return __fdiv_rn(a, __fadd_rn(a, b));
}

// ----------------------------------------------------------- environment
// The envmap emitter of include/optix/light/envmap.h:25-94: direction <->
// (u, v), alias-table pick of a texel followed by a uniform sample of its
// solid angle, and the radiance lookup.  The reference looks radiance up in a
// linear-filtered, wrap-addressed float texture (src/tracer/texture/
// bitmap.cpp:95-99); here the same bilinear filter runs on plain loads with
// fp32 weights.
constexpr float kHalfInvPiF = (float)(0.5 / (double)kPiF);  // (float)(0.5 / M_PIf)

// Bilinear, wrap-addressed lookup at normalised coordinates (u, v) of a
// W x H texel array (the filtering of a CUDA texture with linear filtering
// and wrap addressing, restated with fp32 weights).
__device__ __forceinline__ float3 tex_bilinear(const float4* tex, int W, int H, float u, float v) {
    if (!isfinite(u) || !isfinite(v)) return f3(0.f, 0.f, 0.f);
    u = __fsub_rn(u, floorf(u));
    v = __fsub_rn(v, floorf(v));
    float x = __fsub_rn(__fmul_rn(u, (float)W), 0.5f);
    float y = __fsub_rn(__fmul_rn(v, (float)H), 0.5f);
    float fx = floorf(x), fy = floorf(y);
    float ax = __fsub_rn(x, fx), ay = __fsub_rn(y, fy);
    int x0 = (int)fx, y0 = (int)fy;
    int x1 = x0 + 1, y1 = y0 + 1;
    x0 = x0 < 0 ? x0 + W : x0;
    y0 = y0 < 0 ? y0 + H : y0;
    x1 = x1 >= W ? x1 - W : x1;
    y1 = y1 >= H ? y1 - H : y1;
    float3 t00 = xyz(__ldg(tex + (size_t)y0 * W + x0));
    float3 t10 = xyz(__ldg(tex + (size_t)y0 * W + x1));
    float3 t01 = xyz(__ldg(tex + (size_t)y1 * W + x0));
    float3 t11 = xyz(__ldg(tex + (size_t)y1 * W + x1));
    float bx = __fsub_rn(1.f, ax), by = __fsub_rn(1.f, ay);
    return add(add(add(scale(t00, __fmul_rn(bx, by)), scale(t10, __fmul_rn(ax, by))), scale(t01, __fmul_rn(bx, ay))),
               scale(t11, __fmul_rn(ax, ay)));
}

__device__ __forceinline__ float3 tex_lookup(const DevScene& sc, int t, float2 uv) {
    const DevTexture tx = sc.textures[t];
    return tex_bilinear(tx.texels, tx.w, tx.h, uv.x, uv.y);
}

// Interpolated texture coordinates of a hit (shader_common.h:38-45:
// (1 - u - v) t0 + u t1 + v t2; (0, 0) for a mesh without them).
__device__ __forceinline__ float2 hit_texcoord(const DevScene& sc, int tri, float u, float v) {
    const int4 vi = __ldg(sc.tri_vidx + tri);
    if (!sc.meshes[vi.w].has_texcoords) return make_float2(0.f, 0.f);
    const float2 t0 = __ldg(sc.texcoords + vi.x), t1 = __ldg(sc.texcoords + vi.y), t2 = __ldg(sc.texcoords + vi.z);
    const float b0 = __fsub_rn(__fsub_rn(1.f, u), v);
    return make_float2(__fadd_rn(__fadd_rn(__fmul_rn(b0, t0.x), __fmul_rn(u, t1.x)), __fmul_rn(v, t2.x)),
                       __fadd_rn(__fadd_rn(__fmul_rn(b0, t0.y), __fmul_rn(u, t1.y)), __fmul_rn(v, t2.y)));
}

__device__ __forceinline__ float3 env_lookup(const DevScene& sc, float u, float v) {
    return scale(tex_bilinear(sc.env_tex, sc.env_w, sc.env_h, u, v), sc.env_scale);
}

// Envmap::environment_coords (envmap.h:26-30)
__device__ __forceinline__ float2 env_coords(float3 d) {
    float u = __fadd_rn(__fmul_rn(atan2f(d.z, d.x), kHalfInvPiF), 0.5f);
    float v = __fmul_rn(acosf(fmaxf(fminf(d.y, 1.0f), -1.0f)), kInvPiF);
    return make_float2(u, v);
}

// Envmap::eval (envmap.h:86-91)
__device__ __forceinline__ float3 env_lookup_dir(const DevScene& sc, float3 d) {
    float2 uv = env_coords(d);
    return env_lookup(sc, uv.x, uv.y);
}

// Envmap::pdfDirection (envmap.h:78-84): solid-angle density of the texel.
__device__ __forceinline__ float env_pdf(const DevScene& sc, float3 d) {
    float2 uv = env_coords(d);
    int x = min((int)__fmul_rn(uv.x, (float)sc.env_w), sc.env_w - 1);
    int y = min((int)__fmul_rn(uv.y, (float)sc.env_h), sc.env_h - 1);
    return __ldg(sc.env_accel + (size_t)y * sc.env_w + x).z;
}

// Envmap::sampleDirection (envmap.h:33-76) with three uniform numbers:
// texel pick, alias coin (reused for the position in the texel's phi range),
// position in its cos(theta) range.  Returns radiance * cos / pdf.
__device__ __forceinline__ float3 env_sample(const DevScene& sc, float3 sh_n, float3 xi, float3& d, float& pdf) {
    const unsigned W = (unsigned)sc.env_w, H = (unsigned)sc.env_h, size = W * H;
    unsigned idx = min((unsigned)__fmul_rn(xi.x, (float)size), size - 1u);
    float4 a = __ldg(sc.env_accel + idx);
    unsigned env_idx;
    float xy = xi.y;
    if (xy < a.x) {
        env_idx = idx;
        xy = __fdiv_rn(xy, a.x);
    } else {
        env_idx = __float_as_uint(a.y);
        xy = __fdiv_rn(__fsub_rn(xy, a.x), __fsub_rn(1.0f, a.x));
    }
    const unsigned py = env_idx / W, px = env_idx % W;
    pdf = __ldg(sc.env_accel + env_idx).z;
    float u = __fdiv_rn(__fadd_rn((float)px, xy), (float)W);
    float phi = (float)__dsub_rn(__dmul_rn(__dmul_rn((double)u, 2.0), (double)kPiF), (double)kPiF);
    float step_theta = __fdiv_rn(kPiF, (float)H);
    float theta0 = __fmul_rn((float)py, step_theta);
    float cos_theta = __fadd_rn(__fmul_rn(cosf(theta0), __fsub_rn(1.0f, xi.z)),
                                __fmul_rn(cosf(__fadd_rn(theta0, step_theta)), xi.z));
    float theta = acosf(cos_theta);
    float sin_theta = sinf(theta);
    d = f3(__fmul_rn(cosf(phi), sin_theta), cos_theta, __fmul_rn(sinf(phi), sin_theta));
    if (!(pdf > 0.f)) return f3(0.f, 0.f, 0.f);
    float3 val = env_lookup(sc, u, __fmul_rn(theta, kInvPiF));
    float c = fmaxf(dot(sh_n, d), 0.f);
    return c > 0.f ? divs(scale(val, c), pdf) : f3(0.f, 0.f, 0.f);
}

// ---------------------------------------------------------------- camera
// Row i of a row-major 4x4 matrix times (a0, a1, a2, a3), summed as the
// reference's Matrix4f * Vector4f (include/core/math/matrix.h:265-271 with
// TVector::dot: 0 + a0 m0 + a1 m1 + a2 m2 + a3 m3, left to right).
__device__ __forceinline__ float mrow4(const float* m, int i, float a0, float a1, float a2, float a3) {
    float s = __fadd_rn(0.f, __fmul_rn(a0, m[4 * i]));
    s = __fadd_rn(s, __fmul_rn(a1, m[4 * i + 1]));
    s = __fadd_rn(s, __fmul_rn(a2, m[4 * i + 2]));
    return __fadd_rn(s, __fmul_rn(a3, m[4 * i + 3]));
}

// Camera ray through film position s (pixel units, row 0 = top); tmax is
// the ray's far end (every render ray starts at t = kRayEps).
__device__ __forceinline__ void camera_ray(const DevCamera& c, float2 s, float3& o, float3& d, float& tmax) {
    tmax = __int_as_float(0x7f800000);
    if (c.type == DL_CAMERA_PERSPECTIVE) {
        // perspective.cpp:84-100: near-plane point of the sample, normalised,
        // into world space; the ray spans [near, far] / d.z
        const float sx = __fmul_rn(s.x, c.inv_w), sy = __fmul_rn(s.y, c.inv_h);
        const float w = mrow4(c.S, 3, sx, sy, 0.f, 1.f);
        const float nx = __fdiv_rn(mrow4(c.S, 0, sx, sy, 0.f, 1.f), w);
        const float ny = __fdiv_rn(mrow4(c.S, 1, sx, sy, 0.f, 1.f), w);
        const float nz = __fdiv_rn(mrow4(c.S, 2, sx, sy, 0.f, 1.f), w);
        const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz)));
        const float dx = __fdiv_rn(nx, len), dy = __fdiv_rn(ny, len), dz = __fdiv_rn(nz, len);
        const float ow = mrow4(c.T, 3, 0.f, 0.f, 0.f, 1.f);
        o = f3(__fdiv_rn(mrow4(c.T, 0, 0.f, 0.f, 0.f, 1.f), ow), __fdiv_rn(mrow4(c.T, 1, 0.f, 0.f, 0.f, 1.f), ow),
               __fdiv_rn(mrow4(c.T, 2, 0.f, 0.f, 0.f, 1.f), ow));
        d = f3(mrow4(c.T, 0, dx, dy, dz, 0.f), mrow4(c.T, 1, dx, dy, dz, 0.f), mrow4(c.T, 2, dx, dy, dz, 0.f));
        tmax = __fmul_rn(c.far_clip, __fdiv_rn(1.0f, dz));
        return;
    }
    if (c.type == DL_CAMERA_OPENCV) {
        // include/optix/camera/opencv.h:29-46 with the film position as the
        // pixel sample: (s - c) / f on the z = 1 plane, through the inverse
        // extrinsic, from the eye
        const float px = __fdiv_rn(__fsub_rn(s.x, c.cx), c.fx), py = __fdiv_rn(__fsub_rn(s.y, c.cy), c.fy);
        const float3 head = f3(mrow4(c.T, 0, px, py, 1.f, 1.f), mrow4(c.T, 1, px, py, 1.f, 1.f),
                               mrow4(c.T, 2, px, py, 1.f, 1.f));
        o = ld3(c.eye);
        d = normalize(sub(head, o));
        return;
    }
    float lx = s.x;
    float ly = __fsub_rn(__fsub_rn((float)c.h, s.y), 1.0f);
    float px = __fsub_rn(__fmul_rn(__fmul_rn(lx, c.inv_w), 2.0f), 1.0f);
    float py = __fsub_rn(__fmul_rn(__fmul_rn(ly, c.inv_h), 2.0f), 1.0f);
    d = normalize(add(add(scale(ld3(c.U), px), scale(ld3(c.V), py)), ld3(c.W)));
    o = ld3(c.eye);
}

}  // namespace dl
