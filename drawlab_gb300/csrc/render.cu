// Wavefront path tracer (sm_103a).
//
// The reference runs one path per thread/loop iteration (CPU:
// PathIntegrator::Li, src/tracer/integrator/path.cpp:13-100; OptiX:
// __raygen__path, src/optix/cuda/integrator/path.cu:28-97).  Here a fixed
// pool of path slots advances one segment per iteration through four kernels:
//
//   extend  (queue E[p])  closest hit of every pending ray          -> hit[slot]
//   shadow  (queue S)     any hit of last iteration's NEE rays      -> L[slot] += c
//   retire  (queue R)     paths that ended with a shadow ray in flight: splat,
//                         then start a new camera path in the slot  -> E[q]
//   shade   (queue E[p])  emitter hit + MIS, Russian roulette, NEE (emits a
//                         shadow ray), BSDF sample (emits the next ray) or
//                         finish: splat + new camera path           -> E[q], S, R
//
// Queues are compacted with warp ballots (one atomic per warp).  Every path
// (x, y, s) owns a pcg32 stream and draws its numbers in the reference's order
// (pixel 2D, aperture 2D, then per bounce NEE 2D, BSDF 2D, RR 1D), so each path
// reproduces the oracle's path of the same (x, y, s).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "device.cuh"
#include "internal.h"

namespace dl {

enum PathFlags { PF_CAMERA = 1, PF_PREV_DIFFUSE = 2 };

struct RenderParams {
    DevScene sc;
    float4* ray_o;   // o.xyz, tmin
    float4* ray_d;   // d.xyz, tmax
    float4* hit;     // t, u, v, leaf-order triangle (int bits; -1 = miss)
    float4* tp;      // throughput.rgb, eta
    float4* lacc;    // radiance.rgb, pdf of the last BSDF sample
    int4* meta;      // depth, flags, path index lo, path index hi
    uint4* rng;      // pcg32 state lo/hi, inc lo/hi
    float2* pos;     // film position of the camera sample
    int* ext_q[2];
    int* retire_q;
    float4* sh_o;
    float4* sh_d;
    float4* sh_c;    // contribution.rgb, slot (int bits)
    RenderCounters* cnt;
    float4* film;
    int film_cols, film_rows, border;
    float radius, lookup;
    float filter[33];
    int mode;        // 0: film, 1: Li of explicit paths
    const int* xys;
    float* li_L;
    float* li_pos;
    unsigned long long total_paths;
    int spp_offset;
    int max_depth;
    int rr_depth;
    unsigned int flags;
    unsigned long long seed_mix;
};

// ------------------------------------------------------------ warp helpers
__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// All 32 lanes call this with their predicate; returns the lane's slot in the
// queue (or -1).  One atomic per warp.
__device__ __forceinline__ int warp_push(int* counter, bool pred) {
    unsigned mask = __ballot_sync(0xffffffffu, pred);
    if (mask == 0) return -1;
    int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane_id() == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    return pred ? base + __popc(mask & ((1u << lane_id()) - 1u)) : -1;
}
__device__ __forceinline__ unsigned long long warp_claim(unsigned long long* counter, bool pred) {
    unsigned mask = __ballot_sync(0xffffffffu, pred);
    if (mask == 0) return ~0ull;
    int leader = __ffs(mask) - 1;
    unsigned long long base = 0;
    if (lane_id() == leader) base = atomicAdd(counter, (unsigned long long)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    return pred ? base + (unsigned long long)__popc(mask & ((1u << lane_id()) - 1u)) : ~0ull;
}

__device__ __forceinline__ Pcg32 load_rng(const uint4& r) {
    Pcg32 g;
    g.state = ((uint64_t)r.y << 32) | r.x;
    g.inc = ((uint64_t)r.w << 32) | r.z;
    return g;
}
__device__ __forceinline__ uint4 store_rng(const Pcg32& g) {
    return make_uint4((uint32_t)g.state, (uint32_t)(g.state >> 32), (uint32_t)g.inc, (uint32_t)(g.inc >> 32));
}

// Start path `pid` in `slot`: camera sample and ray (cpu_renderer.cpp:36-44).
__device__ void start_path(const RenderParams& P, int slot, unsigned long long pid) {
    const DevCamera& cam = P.sc.cam;
    int x, y, s;
    if (P.mode == 1) {
        x = P.xys[3 * pid];
        y = P.xys[3 * pid + 1];
        s = P.xys[3 * pid + 2];
    } else {
        unsigned long long npix = (unsigned long long)cam.w * cam.h;
        unsigned long long pix = pid % npix;
        s = (int)(pid / npix) + P.spp_offset;
        x = (int)(pix % cam.w);
        y = (int)(pix / cam.w);
    }
    Pcg32 g;
    seed_path(g, P.seed_mix, cam.w, cam.h, x, y, s);
    float2 ps = g.next2d();
    ps.x = __fadd_rn((float)x, ps.x);
    ps.y = __fadd_rn((float)y, ps.y);
    (void)g.next2d();  // aperture sample: drawn, unused by the "virtual" camera
    float3 o, d;
    camera_ray(cam, ps, o, d);
    P.ray_o[slot] = make_float4(o.x, o.y, o.z, kRayEps);
    P.ray_d[slot] = make_float4(d.x, d.y, d.z, __int_as_float(0x7f800000));
    P.tp[slot] = make_float4(1.f, 1.f, 1.f, 1.f);
    P.lacc[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
    P.meta[slot] = make_int4(0, PF_CAMERA, (int)(pid & 0xffffffffu), (int)(pid >> 32));
    P.rng[slot] = store_rng(g);
    P.pos[slot] = ps;
}

// Film splat (ImageBlock::put, src/core/bitmap/block.cpp:81-113) with float
// atomics into the whole-image film; invalid samples are dropped and counted.
__device__ void splat(const RenderParams& P, float2 pos, float3 v) {
    bool ok = v.x >= 0.f && v.y >= 0.f && v.z >= 0.f && isfinite(v.x) && isfinite(v.y) && isfinite(v.z);
    if (!ok) {
        atomicAdd(&P.cnt->stat_invalid, 1ull);
        return;
    }
    float px = __fsub_rn(__fsub_rn(pos.x, 0.5f), (float)(-P.border));
    float py = __fsub_rn(__fsub_rn(pos.y, 0.5f), (float)(-P.border));
    int x0 = max((int)ceilf(__fsub_rn(px, P.radius)), 0);
    int y0 = max((int)ceilf(__fsub_rn(py, P.radius)), 0);
    int x1 = min((int)floorf(__fadd_rn(px, P.radius)), P.film_cols - 1);
    int y1 = min((int)floorf(__fadd_rn(py, P.radius)), P.film_rows - 1);
    for (int y = y0; y <= y1; y++) {
        float wy = P.filter[min((int)__fmul_rn(fabsf(__fsub_rn((float)y, py)), P.lookup), 32)];
        for (int x = x0; x <= x1; x++) {
            float wx = P.filter[min((int)__fmul_rn(fabsf(__fsub_rn((float)x, px)), P.lookup), 32)];
            float4 c = make_float4(__fmul_rn(__fmul_rn(v.x, wx), wy), __fmul_rn(__fmul_rn(v.y, wx), wy),
                                   __fmul_rn(__fmul_rn(v.z, wx), wy), __fmul_rn(wx, wy));
            atomicAdd(&P.film[(size_t)y * P.film_cols + x], c);
        }
    }
}

// Path `slot` is complete: splat (or write its Li).
__device__ void finish_path(const RenderParams& P, int slot) {
    float4 L = P.lacc[slot];
    if (P.mode == 1) {
        int4 m = P.meta[slot];
        unsigned long long pid = (unsigned long long)(unsigned)m.z | ((unsigned long long)(unsigned)m.w << 32);
        P.li_L[3 * pid] = L.x;
        P.li_L[3 * pid + 1] = L.y;
        P.li_L[3 * pid + 2] = L.z;
        float2 ps = P.pos[slot];
        P.li_pos[2 * pid] = ps.x;
        P.li_pos[2 * pid + 1] = ps.y;
    } else {
        splat(P, P.pos[slot], f3(L.x, L.y, L.z));
    }
}

// Claim new path indices for the lanes in `want`, start them; returns true
// for lanes that now hold a fresh camera ray.
__device__ __forceinline__ bool regenerate(const RenderParams& P, int slot, bool want) {
    unsigned long long pid = warp_claim(&P.cnt->next_path, want);
    bool ok = want && pid < P.total_paths;
    if (ok) start_path(P, slot, pid);
    unsigned mask = __ballot_sync(0xffffffffu, ok);
    if (mask && lane_id() == __ffs(mask) - 1) atomicAdd(&P.cnt->stat_camera, (unsigned long long)__popc(mask));
    return ok;
}

// ---------------------------------------------------------------- kernels
__global__ void k_init(RenderParams P, int capacity) {
    for (int i0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; i0 < capacity;
         i0 += gridDim.x * blockDim.x) {
        int slot = i0 + lane_id();
        bool active = slot < capacity;
        bool ok = regenerate(P, slot, active);
        int e = warp_push(&P.cnt->ext[0], ok);
        if (ok) P.ext_q[0][e] = slot;
    }
}

template <bool kCount>
__global__ void __launch_bounds__(128) k_extend(RenderParams P, int p) {
    int q = p ^ 1;
    int n = P.cnt->ext[p];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        P.cnt->ext[q] = 0;
        P.cnt->shadow[q] = 0;
        P.cnt->retire[q] = 0;
        P.cnt->stat_ext += (unsigned long long)n;
    }
    uint32_t err = 0, nn = 0, nt = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int slot = P.ext_q[p][i];
        float4 o = P.ray_o[slot], d = P.ray_d[slot];
        float t = 0.f, u = 0.f, v = 0.f;
        int tri = trace_closest<kCount>(P.sc, xyz(o), xyz(d), o.w, d.w, t, u, v, err, nn, nt);
        P.hit[slot] = make_float4(t, u, v, __int_as_float(tri));
    }
    if (err) atomicOr(&P.cnt->err, err);
    if (kCount) {
        atomicAdd(&P.cnt->stat_nodes_ext, (unsigned long long)nn);
        atomicAdd(&P.cnt->stat_tris_ext, (unsigned long long)nt);
    }
}

template <bool kCount>
__global__ void __launch_bounds__(128) k_shadow(RenderParams P, int p) {
    int n = P.cnt->shadow[p];
    if (blockIdx.x == 0 && threadIdx.x == 0) P.cnt->stat_shadow += (unsigned long long)n;
    uint32_t err = 0, nn = 0, nt = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 o = P.sh_o[i], d = P.sh_d[i], c = P.sh_c[i];
        if (!trace_any<kCount>(P.sc, xyz(o), xyz(d), o.w, d.w, err, nn, nt)) {
            int slot = __float_as_int(c.w);
            float4 L = P.lacc[slot];
            L.x = __fadd_rn(L.x, c.x);
            L.y = __fadd_rn(L.y, c.y);
            L.z = __fadd_rn(L.z, c.z);
            P.lacc[slot] = L;
        }
    }
    if (err) atomicOr(&P.cnt->err, err);
    if (kCount) {
        atomicAdd(&P.cnt->stat_nodes_sh, (unsigned long long)nn);
        atomicAdd(&P.cnt->stat_tris_sh, (unsigned long long)nt);
    }
}

__global__ void k_retire(RenderParams P, int p) {
    int q = p ^ 1;
    int n = P.cnt->retire[p];
    for (int i0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; i0 < n; i0 += gridDim.x * blockDim.x) {
        int i = i0 + lane_id();
        bool active = i < n;
        int slot = active ? P.retire_q[i] : 0;
        if (active) finish_path(P, slot);
        bool ok = regenerate(P, slot, active);
        int e = warp_push(&P.cnt->ext[q], ok);
        if (ok) P.ext_q[q][e] = slot;
    }
}

struct HitInfo {
    float3 p;
    Frame sh;
    int mesh;
};

__device__ __forceinline__ HitInfo hit_info(const DevScene& sc, int tri, float u, float v) {
    HitInfo h;
    const float4* tp = sc.tris + 3 * tri;
    float3 p0 = xyz(__ldg(tp)), p1 = xyz(__ldg(tp + 1)), p2 = xyz(__ldg(tp + 2));
    float b0 = __fsub_rn(__fsub_rn(1.f, u), v);
    h.p = add(add(scale(p0, b0), scale(p1, u)), scale(p2, v));
    int4 vi = __ldg(sc.tri_vidx + tri);
    h.mesh = vi.w;
    if (sc.meshes[vi.w].has_normals) {
        float3 n0 = xyz(__ldg(sc.normals + vi.x)), n1 = xyz(__ldg(sc.normals + vi.y));
        float3 n2 = normalize(xyz(__ldg(sc.normals + vi.z)));
        // only the third term normalised (src/tracer/accel/octree.cpp:202-206)
        h.sh = make_frame(add(add(scale(n0, b0), scale(n1, u)), scale(n2, v)));
    } else {
        h.sh = make_frame(normalize(cross(sub(p1, p0), sub(p2, p0))));
    }
    return h;
}

// Mesh::samplePosition over an area light's triangles (mesh.cpp:222-244,
// DiscretePDF::sampleReuse dpdf.h:131-136).
__device__ __forceinline__ void sample_area(const DevScene& sc, const DevLight& L, float2 s, float3& p,
                                            float3& n) {
    const float* cdf = sc.emit_cdf + L.cdf_begin;
    int cnt = L.tri_count;
    // lower_bound over cdf[0..cnt]
    int lo = 0, hi = cnt + 1;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (__ldg(cdf + mid) < s.x) lo = mid + 1; else hi = mid;
    }
    int f = max(lo - 1, 0);
    f = min(f, cnt - 1);
    float c0 = __ldg(cdf + f), c1 = __ldg(cdf + f + 1);
    s.x = __fdiv_rn(__fsub_rn(s.x, c0), __fsub_rn(c1, c0));
    const float4* et = sc.emit_tris + 6 * (L.tri_begin + f);
    float3 p0 = xyz(__ldg(et)), p1 = xyz(__ldg(et + 1)), p2 = xyz(__ldg(et + 2));
    float3 b = square_to_uniform_triangle(s);
    p = add(add(scale(p0, b.x), scale(p1, b.y)), scale(p2, b.z));
    if (L.has_normals) {
        float3 n0 = xyz(__ldg(et + 3)), n1 = xyz(__ldg(et + 4)), n2 = xyz(__ldg(et + 5));
        n = add(add(scale(n0, b.x), scale(n1, b.y)), scale(n2, b.z));
    } else {
        n = cross(sub(p1, p0), sub(p2, p1));
    }
    n = normalize(n);
}

// Scene::sampleEmitterDirection without the visibility test (the caller
// traces the shadow ray).  Returns the unoccluded spectrum.
__device__ __forceinline__ float3 sample_emitter(const RenderParams& P, float3 its_p, float3 sh_n, float2 s,
                                                 float3& d, float& dist, float& pdf, bool& delta) {
    const DevScene& sc = P.sc;
    int N = sc.num_lights;
    float3 zero = f3(0.f, 0.f, 0.f);
    delta = false;
    pdf = 0.f;
    dist = 0.f;
    d = zero;
    if (N == 0) return zero;
    int idx = 0;
    if (N > 1) {
        float fn = (float)N;
        idx = min((int)__fmul_rn(s.x, fn), N - 1);
        s.x = __fsub_rn(__fmul_rn(s.x, fn), (float)idx);
    }
    const DevLight& L = sc.lights[idx];
    float3 spec;
    if (L.type == LIGHT_AREA) {
        float3 lp, ln;
        sample_area(sc, L, s, lp, ln);
        float3 vec = sub(lp, its_p);
        d = normalize(vec);
        dist = length(vec);
        float dp = fmaxf(dot(ln, neg(d)), 0.f);
        float pw = dp != 0.f ? __fdiv_rn(__fmul_rn(__fmul_rn(L.pA, dist), dist), dp) : 0.f;
        pdf = pw;
        spec = pw != 0.f ? divs(scale(ld3(L.radiance), fmaxf(dot(sh_n, d), 0.f)), pw) : zero;
    } else if (L.type == LIGHT_POINT) {
        float3 vec = sub(ld3(L.position), its_p);
        d = normalize(vec);
        dist = length(vec);
        pdf = 1.f;
        delta = true;
        float inv = __fdiv_rn(1.0f, dist);
        if (P.flags & DL_RENDER_FIX_POINT_LIGHT) {
            float c = fmaxf(dot(sh_n, d), 0.f);
            spec = c > 0.f ? scale(scale(scale(ld3(L.radiance), c), inv), inv) : zero;
        } else {
            spec = scale(scale(ld3(L.radiance), inv), inv);
        }
    } else {
        spec = zero;
    }
    if (N > 1) {
        spec = scale(spec, (float)N);
        pdf = __fmul_rn(pdf, __fdiv_rn(1.f, (float)N));
    }
    return spec;
}

__global__ void __launch_bounds__(128) k_shade(RenderParams P, int p) {
    const int q = p ^ 1;
    const DevScene& sc = P.sc;
    int n = P.cnt->ext[p];
    for (int i0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; i0 < n; i0 += gridDim.x * blockDim.x) {
        int i = i0 + lane_id();
        bool active = i < n;
        int slot = active ? P.ext_q[p][i] : 0;
        bool cont = false, emit_shadow = false, finish = false;
        float4 sh_o = make_float4(0.f, 0.f, 0.f, 0.f), sh_d = sh_o, sh_c = sh_o;
        if (active) {
            float4 hit = P.hit[slot];
            int tri = __float_as_int(hit.w);
            float4 ro = P.ray_o[slot], rd = P.ray_d[slot];
            float4 tpe = P.tp[slot];
            float4 L = P.lacc[slot];
            int4 meta = P.meta[slot];
            float3 tp = f3(tpe.x, tpe.y, tpe.z);
            float eta = tpe.w;
            float3 Lr = f3(L.x, L.y, L.z);
            float prev_pdf = L.w;
            int depth = meta.x;
            int flags = meta.y;
            Pcg32 g = load_rng(P.rng[slot]);
            bool done = false;
            HitInfo h;
            float3 dir = xyz(rd);
            if (tri < 0) {
                done = true;  // miss: path.cpp:23-25 / 85-87
            } else {
                h = hit_info(sc, tri, hit.y, hit.z);
                int light = sc.meshes[h.mesh].light;
                if (flags & PF_CAMERA) {
                    if (light >= 0) {
                        // first hit: emission without MIS (path.cpp:27-29)
                        const DevLight& Lt = sc.lights[light];
                        if (dot(h.sh.n, neg(dir)) > 0.f) Lr = add(Lr, mul(tp, ld3(Lt.radiance)));
                    }
                    depth = 0;
                } else {
                    if (light >= 0) {
                        // BSDF-sampled ray hit an emitter (path.cpp:72-84)
                        const DevLight& Lt = sc.lights[light];
                        float3 le = dot(h.sh.n, neg(dir)) > 0.f ? ld3(Lt.radiance) : f3(0.f, 0.f, 0.f);
                        float3 vec = sub(h.p, xyz(ro));
                        float3 dd = normalize(vec);
                        float dist = length(vec);
                        float dp = fmaxf(dot(h.sh.n, neg(dd)), 0.f);
                        float ep = dp != 0.f ? __fdiv_rn(__fmul_rn(__fmul_rn(Lt.pA, dist), dist), dp) : 0.f;
                        if (sc.num_lights != 1) ep = __fdiv_rn(ep, (float)sc.num_lights);
                        float w = (flags & PF_PREV_DIFFUSE) ? mis_weight(prev_pdf, ep) : 1.f;
                        Lr = add(Lr, mul(scale(tp, w), le));
                    }
                    // Russian roulette (path.cpp:89-97)
                    if (depth > P.rr_depth) {
                        float pr = fminf(maxc(scale(scale(tp, eta), eta)), 0.99f);
                        if (g.next_float() > pr) done = true;
                        else tp = divs(tp, pr);
                    }
                    depth += 1;
                }
                if (!done && P.max_depth > 0 && depth >= P.max_depth) done = true;
            }
            if (!done) {
                const DevMaterial& m = sc.materials[sc.meshes[h.mesh].material];
                bool aniso = m.type == MAT_ANISO_GGX;
                Frame fr = aniso ? make_onb(normalize(h.sh.n)) : h.sh;
                // ---- emitter sampling (path.cpp:36-56)
                float2 s_nee = g.next2d();
                float3 ld;
                float ldist, lpdf;
                bool delta;
                float3 espec = sample_emitter(P, h.p, h.sh.n, s_nee, ld, ldist, lpdf, delta);
                float3 wi = to_local(fr, neg(normalize(dir)));
                if (aniso) wi = normalize(wi);
                if (__fadd_rn(__fadd_rn(espec.x, espec.y), espec.z) > 0.f && lpdf > 0.f) {
                    BRec q1;
                    q1.wi = wi;
                    q1.wo = to_local(fr, ld);
                    q1.measure = M_SOLID;
                    q1.eta = 1.f;
                    float3 bv = bsdf_eval(m, q1);
                    float bp = bsdf_pdf(m, q1);
                    float w = (delta && (P.flags & DL_RENDER_FIX_POINT_LIGHT)) ? 1.f : mis_weight(lpdf, bp);
                    float3 c = mul(mul(scale(tp, w), bv), espec);
                    if (c.x != 0.f || c.y != 0.f || c.z != 0.f) {
                        emit_shadow = true;
                        sh_o = make_float4(h.p.x, h.p.y, h.p.z, kRayEps);
                        sh_d = make_float4(ld.x, ld.y, ld.z, __fsub_rn(ldist, kRayEps));
                        sh_c = make_float4(c.x, c.y, c.z, __int_as_float(slot));
                    }
                }
                // ---- BSDF sampling (path.cpp:60-69)
                BRec q2;
                q2.wi = wi;
                q2.wo = f3(0.f, 0.f, 0.f);
                q2.eta = 1.f;
                q2.measure = M_UNKNOWN;
                float3 f = bsdf_sample(m, q2, g.next2d());
                tp = mul(tp, f);
                eta = __fmul_rn(eta, q2.eta);
                prev_pdf = bsdf_pdf(m, q2);
                flags = is_diffuse(m.type) ? PF_PREV_DIFFUSE : 0;
                float3 nd = to_world(fr, q2.wo);
                if (aniso) nd = normalize(nd);
                if (tp.x == 0.f && tp.y == 0.f && tp.z == 0.f) {
                    done = true;  // every later contribution is zero
                } else {
                    P.ray_o[slot] = make_float4(h.p.x, h.p.y, h.p.z, kRayEps);
                    P.ray_d[slot] = make_float4(nd.x, nd.y, nd.z, __int_as_float(0x7f800000));
                    cont = true;
                }
            }
            P.tp[slot] = make_float4(tp.x, tp.y, tp.z, eta);
            P.lacc[slot] = make_float4(Lr.x, Lr.y, Lr.z, prev_pdf);
            P.meta[slot] = make_int4(depth, flags, meta.z, meta.w);
            P.rng[slot] = store_rng(g);
            finish = done && !emit_shadow;
        }
        bool retire = active && !cont && emit_shadow;
        int sp = warp_push(&P.cnt->shadow[q], emit_shadow);
        if (emit_shadow) {
            P.sh_o[sp] = sh_o;
            P.sh_d[sp] = sh_d;
            P.sh_c[sp] = sh_c;
        }
        int rp = warp_push(&P.cnt->retire[q], retire);
        if (retire) P.retire_q[rp] = slot;
        if (finish) finish_path(P, slot);
        bool fresh = regenerate(P, slot, finish);
        bool push = cont || fresh;
        int e = warp_push(&P.cnt->ext[q], push);
        if (push) P.ext_q[q][e] = slot;
    }
}

// film -> rgb (ImageBlock::toBitmap, block.cpp:58-66)
__global__ void k_resolve(const float4* film, int cols, int border, int w, int h, float* rgb) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    int x = i % w, y = i / w;
    float4 c = film[(size_t)(y + border) * cols + (x + border)];
    float r = 0.f, g = 0.f, b = 0.f;
    if (c.w != 0.f) {
        r = __fdiv_rn(c.x, c.w);
        g = __fdiv_rn(c.y, c.w);
        b = __fdiv_rn(c.z, c.w);
    }
    rgb[3 * (size_t)i] = r;
    rgb[3 * (size_t)i + 1] = g;
    rgb[3 * (size_t)i + 2] = b;
}

// ------------------------------------------------------------------- host
void RenderBuffers::ensure(int64_t cap) {
    if (cap <= capacity) return;
    size_t c = (size_t)cap;
    ray_o.ensure(16 * c);
    ray_d.ensure(16 * c);
    hit.ensure(16 * c);
    tp.ensure(16 * c);
    lacc.ensure(16 * c);
    meta.ensure(16 * c);
    rng.ensure(16 * c);
    pos.ensure(8 * c);
    ext_q[0].ensure(4 * c);
    ext_q[1].ensure(4 * c);
    retire_q.ensure(4 * c);
    sh_o.ensure(16 * c);
    sh_d.ensure(16 * c);
    sh_c.ensure(16 * c);
    counters.ensure(sizeof(RenderCounters));
    host_counters.ensure(sizeof(RenderCounters));
    capacity = cap;
}

size_t RenderBuffers::device_bytes() const {
    return ray_o.bytes + ray_d.bytes + hit.bytes + tp.bytes + lacc.bytes + meta.bytes + rng.bytes +
           pos.bytes + ext_q[0].bytes + ext_q[1].bytes + retire_q.bytes + sh_o.bytes + sh_d.bytes +
           sh_c.bytes + counters.bytes + film.bytes + rgb.bytes;
}

void filter_setup(int filter, float& radius, int& border, float& lookup, float* table) {
    const int RES = 32;
    radius = filter == DL_FILTER_BOX ? 0.5f : 2.0f;
    border = (int)std::ceil(radius - 0.5f);
    for (int i = 0; i < RES; ++i) {
        float pos = (radius * i) / RES;
        if (filter == DL_FILTER_BOX) {
            table[i] = 1.0f;
        } else {
            const float stddev = 0.5f;
            float alpha = -1.0f / (2.0f * stddev * stddev);
            table[i] = std::max(0.0f, std::exp(alpha * pos * pos) - std::exp(alpha * radius * radius));
        }
    }
    table[RES] = 0.0f;
    lookup = RES / radius;
}

int64_t film_floats(int w, int h, int filter) {
    int b = filter == DL_FILTER_BOX ? 0 : 2;
    return (int64_t)(w + 2 * b) * (h + 2 * b) * 4;
}

// Runs one render.  mode 0: splat into d_film (zeroed here); mode 1: Li of
// li_n explicit paths (d_xys -> d_L, d_pos).
void render_run(dl_scene* S, const dl_render_opts& o, float* d_film, int64_t li_n, const int* d_xys,
                float* d_L, float* d_pos, bool count_traversal, RenderCounters* out_counters) {
    dl_context* ctx = S->ctx;
    cudaStream_t st = ctx->stream;
    const DevCamera& cam = S->dev.cam;
    RenderParams P;
    std::memset(&P, 0, sizeof(P));
    P.sc = S->dev;
    P.mode = li_n > 0 ? 1 : 0;
    unsigned long long total =
        P.mode == 1 ? (unsigned long long)li_n : (unsigned long long)cam.w * cam.h * (unsigned long long)std::max(o.spp, 0);
    int64_t cap = o.max_paths_in_flight > 0 ? o.max_paths_in_flight : (int64_t)1 << 22;
    cap = std::min<int64_t>(cap, (int64_t)std::max<unsigned long long>(total, 1ull));
    cap = ((cap + 31) / 32) * 32;
    RenderBuffers& B = ctx->render;
    B.ensure(cap);
    P.ray_o = B.ray_o.as<float4>();
    P.ray_d = B.ray_d.as<float4>();
    P.hit = B.hit.as<float4>();
    P.tp = B.tp.as<float4>();
    P.lacc = B.lacc.as<float4>();
    P.meta = B.meta.as<int4>();
    P.rng = B.rng.as<uint4>();
    P.pos = B.pos.as<float2>();
    P.ext_q[0] = B.ext_q[0].as<int>();
    P.ext_q[1] = B.ext_q[1].as<int>();
    P.retire_q = B.retire_q.as<int>();
    P.sh_o = B.sh_o.as<float4>();
    P.sh_d = B.sh_d.as<float4>();
    P.sh_c = B.sh_c.as<float4>();
    P.cnt = B.counters.as<RenderCounters>();
    filter_setup(o.filter, P.radius, P.border, P.lookup, P.filter);
    P.film_cols = cam.w + 2 * P.border;
    P.film_rows = cam.h + 2 * P.border;
    P.film = reinterpret_cast<float4*>(d_film);
    P.xys = d_xys;
    P.li_L = d_L;
    P.li_pos = d_pos;
    P.total_paths = total;
    P.spp_offset = o.spp_offset;
    P.max_depth = o.max_depth;
    P.rr_depth = o.rr_depth;
    P.flags = o.flags;
    P.seed_mix = splitmix64(o.seed);

    if (P.mode == 0) DL_CUDA(cudaMemsetAsync(d_film, 0, sizeof(float) * film_floats(cam.w, cam.h, o.filter), st));
    DL_CUDA(cudaMemsetAsync(P.cnt, 0, sizeof(RenderCounters), st));
    const int sms = ctx->num_sms > 0 ? ctx->num_sms : 152;
    const int trace_blocks = sms * 16, trace_threads = 128;
    const int work_blocks = sms * 16, work_threads = 128;
    // Optional per-kernel timing: one event pair per launch, four kernels per
    // iteration, read back at every counter check.
    const int check_every = 4;
    const bool timing = ctx->kernel_timing;
    if (timing && ctx->timing_events.empty()) {
        ctx->timing_events.resize(2 * 4 * check_every);
        for (auto& e : ctx->timing_events) DL_CUDA(cudaEventCreate(&e));
    }
    double kms[4] = {0, 0, 0, 0};
    int64_t launches = 1;
    DL_CUDA(cudaEventRecord(ctx->ev0, st));
    k_init<<<work_blocks, work_threads, 0, st>>>(P, (int)cap);
    RenderCounters* hc = B.host_counters.as<RenderCounters>();
    int64_t iters = 0;
    for (;;) {
        for (int k = 0; k < check_every; k++) {
            int p = (int)(iters & 1);
            cudaEvent_t* ev = timing ? &ctx->timing_events[8 * k] : nullptr;
            if (timing) DL_CUDA(cudaEventRecord(ev[0], st));
            if (count_traversal) k_extend<true><<<trace_blocks, trace_threads, 0, st>>>(P, p);
            else k_extend<false><<<trace_blocks, trace_threads, 0, st>>>(P, p);
            if (timing) DL_CUDA(cudaEventRecord(ev[1], st));
            if (timing) DL_CUDA(cudaEventRecord(ev[2], st));
            if (count_traversal) k_shadow<true><<<trace_blocks, trace_threads, 0, st>>>(P, p);
            else k_shadow<false><<<trace_blocks, trace_threads, 0, st>>>(P, p);
            if (timing) DL_CUDA(cudaEventRecord(ev[3], st));
            if (timing) DL_CUDA(cudaEventRecord(ev[4], st));
            k_retire<<<work_blocks, work_threads, 0, st>>>(P, p);
            if (timing) DL_CUDA(cudaEventRecord(ev[5], st));
            if (timing) DL_CUDA(cudaEventRecord(ev[6], st));
            k_shade<<<work_blocks, work_threads, 0, st>>>(P, p);
            if (timing) DL_CUDA(cudaEventRecord(ev[7], st));
            iters++;
            launches += 4;
        }
        DL_CUDA(cudaGetLastError());
        DL_CUDA(cudaMemcpyAsync(hc, P.cnt, sizeof(RenderCounters), cudaMemcpyDeviceToHost, st));
        DL_CUDA(cudaStreamSynchronize(st));
        if (timing) {
            for (int k = 0; k < check_every; k++)
                for (int j = 0; j < 4; j++) {
                    float ms = 0.f;
                    DL_CUDA(cudaEventElapsedTime(&ms, ctx->timing_events[8 * k + 2 * j],
                                                 ctx->timing_events[8 * k + 2 * j + 1]));
                    kms[j] += ms;
                }
        }
        int p = (int)(iters & 1);
        if (hc->err) throw Error(DL_ERR_QUEUE_OVERFLOW, "traversal stack overflow");
        if (hc->ext[p] == 0 && hc->shadow[p] == 0 && hc->retire[p] == 0 && hc->next_path >= total) break;
        if (iters > 1000000) throw Error(DL_ERR_TIMEOUT, "render did not converge");
    }
    ctx->stats.extend_ms = kms[0];
    ctx->stats.shadow_ms = kms[1];
    ctx->stats.retire_ms = kms[2];
    ctx->stats.shade_ms = kms[3];
    ctx->stats.kernel_launches = launches;
    DL_CUDA(cudaEventRecord(ctx->ev1, st));
    DL_CUDA(cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    DL_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->stats.camera_rays = (int64_t)hc->stat_camera;
    ctx->stats.extension_rays = (int64_t)hc->stat_ext;
    ctx->stats.shadow_rays = (int64_t)hc->stat_shadow;
    ctx->stats.invalid_samples = (int64_t)hc->stat_invalid;
    ctx->stats.iterations = iters;
    ctx->stats.render_ms = ms;
    if (out_counters) *out_counters = *hc;
}

// Li of explicit paths with every piece of path state in caller-provided
// device memory (`pool`, laid out by fixed_pool_layout) and no allocation of
// any kind: no cudaMalloc, no pinned staging (the counters are read back into
// a stack copy), no exceptions.  Used by the allocation-free entry point.
size_t fixed_pool_bytes(int64_t slots) {
    size_t c = (size_t)slots;
    return 7 * 16 * c + 8 * c + 3 * 4 * c + 3 * 16 * c + 256;
}

cudaError_t render_li_fixed(dl_scene* S, const dl_render_opts& o, void* pool, int64_t slots, int64_t li_n,
                            const int* d_xys, float* d_L, float* d_pos) {
    dl_context* ctx = S->ctx;
    cudaStream_t st = ctx->stream;
    RenderParams P;
    std::memset(&P, 0, sizeof(P));
    P.sc = S->dev;
    P.mode = 1;
    size_t c = (size_t)slots;
    char* b = static_cast<char*>(pool);
    P.cnt = reinterpret_cast<RenderCounters*>(b);
    b += 256;
    P.ray_o = reinterpret_cast<float4*>(b); b += 16 * c;
    P.ray_d = reinterpret_cast<float4*>(b); b += 16 * c;
    P.hit = reinterpret_cast<float4*>(b); b += 16 * c;
    P.tp = reinterpret_cast<float4*>(b); b += 16 * c;
    P.lacc = reinterpret_cast<float4*>(b); b += 16 * c;
    P.meta = reinterpret_cast<int4*>(b); b += 16 * c;
    P.rng = reinterpret_cast<uint4*>(b); b += 16 * c;
    P.sh_o = reinterpret_cast<float4*>(b); b += 16 * c;
    P.sh_d = reinterpret_cast<float4*>(b); b += 16 * c;
    P.sh_c = reinterpret_cast<float4*>(b); b += 16 * c;
    P.pos = reinterpret_cast<float2*>(b); b += 8 * c;
    P.ext_q[0] = reinterpret_cast<int*>(b); b += 4 * c;
    P.ext_q[1] = reinterpret_cast<int*>(b); b += 4 * c;
    P.retire_q = reinterpret_cast<int*>(b);
    filter_setup(o.filter, P.radius, P.border, P.lookup, P.filter);
    P.film_cols = S->dev.cam.w + 2 * P.border;
    P.film_rows = S->dev.cam.h + 2 * P.border;
    P.xys = d_xys;
    P.li_L = d_L;
    P.li_pos = d_pos;
    P.total_paths = (unsigned long long)li_n;
    P.max_depth = o.max_depth;
    P.rr_depth = o.rr_depth;
    P.flags = o.flags;
    P.seed_mix = splitmix64(o.seed);
    int64_t cap = std::min<int64_t>(slots, ((li_n + 31) / 32) * 32);
    const int sms = ctx->num_sms > 0 ? ctx->num_sms : 152;
    cudaError_t e = cudaMemsetAsync(P.cnt, 0, sizeof(RenderCounters), st);
    if (e != cudaSuccess) return e;
    k_init<<<sms * 16, 128, 0, st>>>(P, (int)cap);
    RenderCounters hc;
    int64_t iters = 0;
    for (;;) {
        for (int k = 0; k < 4; k++) {
            int p = (int)(iters & 1);
            k_extend<false><<<sms * 16, 128, 0, st>>>(P, p);
            k_shadow<false><<<sms * 16, 128, 0, st>>>(P, p);
            k_retire<<<sms * 16, 128, 0, st>>>(P, p);
            k_shade<<<sms * 16, 128, 0, st>>>(P, p);
            iters++;
        }
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(&hc, P.cnt, sizeof(RenderCounters), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
        int p = (int)(iters & 1);
        if (hc.err) return cudaErrorUnknown;
        if (hc.ext[p] == 0 && hc.shadow[p] == 0 && hc.retire[p] == 0 && hc.next_path >= (unsigned long long)li_n) break;
        if (iters > 1000000) return cudaErrorLaunchTimeout;
    }
    return cudaSuccess;
}

void resolve_film(dl_scene* S, const float* d_film, int filter, float* d_rgb) {
    const DevCamera& cam = S->dev.cam;
    int b = filter == DL_FILTER_BOX ? 0 : 2;
    int n = cam.w * cam.h;
    k_resolve<<<(n + 255) / 256, 256, 0, S->ctx->stream>>>(reinterpret_cast<const float4*>(d_film),
                                                         cam.w + 2 * b, b, cam.w, cam.h, d_rgb);
    DL_CUDA(cudaGetLastError());
}

}  // namespace dl
