// Wavefront path tracer (sm_103a).
//
// The reference runs one path per thread/loop iteration (CPU:
// PathIntegrator::Li, src/tracer/integrator/path.cpp:13-100; OptiX:
// __raygen__path, src/optix/cuda/integrator/path.cu:28-97).  Here a fixed
// pool of path slots advances one segment per iteration through:
//
//   extend    persistent closest-hit traversal of queue E[p]; lanes whose ray
//             finishes fetch the next one (per-lane replacement); each hit
//             joins the queue of its material type, misses the miss queue
//   shadow    same, any hit, for last iteration's NEE rays: the contribution
//             goes to the path (or, if the path has ended, to its sample)
//   miss      paths whose ray missed: store the sample, start a new camera
//             path in the slot                                     -> E[q]
//   material  one kernel per BSDF type (diffuse, mirror, dielectric,
//             Beckmann microfacet, GGX): emitter hit + MIS, Russian roulette,
//             NEE (emits a shadow ray), BSDF sampling (emits the next ray);
//             a path that ends stores its sample and its slot starts a new
//             camera path                                          -> E[q], S
//   film      after the last path: gather every sample into the film
//
// Path state lives in 32-byte records (ray, path, meta+rng, hit), each read
// and written whole: a full DRAM sector, no read-modify-write of partial
// sectors.  Queues are compacted with warp ballots: one atomic per warp, or
// per 32 entries where a warp stages them in shared memory; the hot counters
// sit in separate 128-byte lines.  A
// batch of iterations is captured once as a CUDA graph and replayed.  Every
// path (x, y, s) owns a pcg32 stream and draws its numbers in the reference's
// order (pixel 2D, aperture 2D, then per bounce NEE 2D, BSDF 2D, RR 1D), so
// each path reproduces the oracle's path of the same (x, y, s).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>

#include "device.cuh"
#include "guide.cuh"
#include "guide_tc.cuh"
#include "internal.h"
#include "scene.h"

namespace dl {

enum PathFlags { PF_CAMERA = 1, PF_PREV_DIFFUSE = 2 };

struct __align__(32) RayRec {
    float4 o;   // origin, tmin
    float4 d;   // direction, tmax
};
struct __align__(32) PathRec {
    float4 tp;  // throughput.rgb, eta
    float4 L;   // radiance.rgb, pdf of the last BSDF sample
};
struct __align__(32) MetaRec {
    int4 m;     // depth, flags, path index lo, path index hi
    uint4 rng;  // pcg32 state lo/hi, inc lo/hi
};
struct __align__(32) HitRec {
    float4 h;   // t, u, v, leaf-order triangle (int bits; -1 = miss)
    float4 pad;
};
static_assert(sizeof(RayRec) == 32 && sizeof(PathRec) == 32 && sizeof(MetaRec) == 32 && sizeof(HitRec) == 32,
              "path records are one 32-byte sector each");
// A slot's four records share one 128-byte line: the ray and its hit in one
// half, the path state in the other.  Slots are visited in queue order, i.e.
// at random; a random 32-byte read costs a whole DRAM burst, so records read
// together are kept inside one.
struct __align__(128) SlotRec {
    RayRec ray;
    HitRec hit;
    PathRec path;
    MetaRec meta;
};
static_assert(sizeof(SlotRec) == 128, "one 128-byte line per slot");
constexpr size_t kSlotBytes = 4 * 32 + 8 + 3 * 16 + 4 * (2 + kNumMaterialTypes + 1);  // records, pos, shadow, queues

constexpr int kMissQueue = kNumMaterialTypes;  // queue index of rays that hit nothing

// One render request: a scene and its render options.  A single render has
// one request, carried in the kernel parameters; a batch has a table of them
// in device memory and every path carries its request's index (in the path
// flags, in the ray records' w slot).
struct DevRequest {
    DevScene sc;
    unsigned long long pid_first;  // the request's first path index in the current pass
    int spp_offset;                // sample index of its first sample in the pass
    int max_depth;
    int rr_depth;
    unsigned int flags;
    unsigned long long seed_mix;
};
constexpr int kReqShift = 8;  // path flags: request index << kReqShift | PathFlags

// Guided renders: per slot, the training records of the path's two most
// recent guided vertices with the throughput after each (a: older, b: newer;
// record index in w, -1 for none).  Radiance the path gathers later is
// credited to them divided by that throughput: the estimate of the radiance
// arriving along the direction sampled there.
struct __align__(32) GuideRec {
    float4 a;
    float4 b;
};

struct RenderParams {
    DevRequest r0;                 // the request of a single render
    int capacity;                  // path slots (queue and record arrays hold this many entries)
    const DevRequest* reqs;        // batch: request table (pid_first ascending)
    int num_reqs;
    SlotRec* rec;    // per slot: ray, hit, path state
    float2* pos;     // film position of the camera sample (Li mode only)
    int* ext_q[2];
    int* mat_q[kNumMaterialTypes + 1];  // per material type, then the miss queue
    float4* sh_o;
    float4* sh_d;
    float4* sh_c;    // contribution.rgb, target: slot >= 0 (live path) or -1 - path index (ended path)
    RenderCounters* cnt;
    float4* samples; // radiance.rgb + presence flag per path index of this chunk
    int mode;        // 0: film, 1: Li of explicit paths
    const int* xys;
    float* li_L;
    float* li_pos;
    // guided renders
    int guided;
    GuideNet gnet;
    GuideRec* grec;
    GuideRecord* grecords;
    int grecord_cap;
};

template <bool kMulti>
__device__ __forceinline__ const DevRequest& request(const RenderParams& P, int rid) {
    if (kMulti) return P.reqs[rid];
    return P.r0;
}

// Bounds-checked build (compiled with -DDL_CHECKS): before each access whose
// index comes from a queue, a counter or a record -- path slots, queue
// positions, path indices, BVH nodes and triangles -- the index is checked
// against its array; a violation sets kErrBounds in the render's error word
// and the access is skipped.  Without DL_CHECKS the checks compile to
// nothing.
constexpr unsigned kErrBounds = 4u;
#ifdef DL_CHECKS
__device__ __forceinline__ bool in_bounds(bool ok, unsigned int* err) {
    if (!ok) atomicOr(err, kErrBounds);
    return ok;
}
#define DL_IN_BOUNDS(cond, err) in_bounds((cond), (err))
#else
#define DL_IN_BOUNDS(cond, err) true
#endif
constexpr const char* kBoundsMessage = "bounds check failed: a queue, slot, path, node or triangle index "
                                        "outside its array (bounds-checked build)";
// 32 bytes (32-byte aligned) of read-only global data in one load.
__device__ __forceinline__ void ld_nc_256(const float4* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}
__device__ __forceinline__ bool slot_ok(const RenderParams& P, int slot) {
    return DL_IN_BOUNDS(slot >= 0 && slot < P.capacity, &P.cnt->err);
}

// Request of batch path `pid`: the last request whose first path is <= pid.
__device__ __forceinline__ int find_request(const RenderParams& P, unsigned long long pid) {
    int lo = 0, hi = P.num_reqs;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (P.reqs[mid].pid_first <= pid) lo = mid; else hi = mid;
    }
    return lo;
}

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

__device__ __forceinline__ unsigned long long warp_claim_u32(unsigned int* counter, bool pred) {
    unsigned mask = __ballot_sync(0xffffffffu, pred);
    if (mask == 0) return ~0ull;
    int leader = __ffs(mask) - 1;
    unsigned base = 0;
    if (lane_id() == leader) base = atomicAdd(counter, (unsigned)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    return pred ? (unsigned long long)base + __popc(mask & ((1u << lane_id()) - 1u)) : ~0ull;
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
__device__ __forceinline__ unsigned long long path_index(const int4& m) {
    return (unsigned long long)(unsigned)m.z | ((unsigned long long)(unsigned)m.w << 32);
}

// Start path `pid` in `slot`: camera sample and ray (cpu_renderer.cpp:36-44).
// Ray records carry the request index in o.w (every render ray starts at
// tmin = kRayEps).
template <bool kMulti>
__device__ void start_path(const RenderParams& P, int slot, unsigned long long pid) {
    if (!slot_ok(P, slot) || !DL_IN_BOUNDS(pid < P.cnt->pass_total, &P.cnt->err)) return;
    const int rid = kMulti ? find_request(P, pid) : 0;
    const DevRequest& R = request<kMulti>(P, rid);
    const DevCamera& cam = R.sc.cam;
    int x, y, s;
    if (P.mode == 1) {
        x = P.xys[3 * pid];
        y = P.xys[3 * pid + 1];
        s = P.xys[3 * pid + 2];
    } else {
        unsigned long long local = pid - R.pid_first;
        unsigned long long npix = (unsigned long long)cam.w * cam.h;
        if ((local | npix) < 0x100000000ull) {  // 32-bit division where it fits
            const unsigned l32 = (unsigned)local, n32 = (unsigned)npix, pix = l32 % n32;
            s = (int)(l32 / n32);
            x = (int)(pix % (unsigned)cam.w);
            y = (int)(pix / (unsigned)cam.w);
        } else {
            unsigned long long pix = local % npix;
            s = (int)(local / npix);
            x = (int)(pix % cam.w);
            y = (int)(pix / cam.w);
        }
        s += kMulti ? R.spp_offset : P.cnt->pass_spp_offset;
    }
    Pcg32 g;
    seed_path(g, R.seed_mix, cam.w, cam.h, x, y, s);
    float2 ps = g.next2d();
    ps.x = __fadd_rn((float)x, ps.x);
    ps.y = __fadd_rn((float)y, ps.y);
    (void)g.next2d();  // aperture sample: drawn, unused by the "virtual" camera
    float3 o, d;
    float tmax;
    camera_ray(cam, ps, o, d, tmax);
    RayRec r;
    r.o = make_float4(o.x, o.y, o.z, __int_as_float(rid));
    r.d = make_float4(d.x, d.y, d.z, tmax);
    P.rec[slot].ray = r;
    PathRec pr;
    pr.tp = make_float4(1.f, 1.f, 1.f, 1.f);
    pr.L = make_float4(0.f, 0.f, 0.f, 0.f);
    P.rec[slot].path = pr;
    MetaRec mr;
    mr.m = make_int4(0, PF_CAMERA | (rid << kReqShift), (int)(pid & 0xffffffffu), (int)(pid >> 32));
    mr.rng = store_rng(g);
    P.rec[slot].meta = mr;
    if (P.mode == 1) P.pos[slot] = ps;
    if (P.guided) {
        GuideRec gr;
        gr.a = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
        gr.b = gr.a;
        P.grec[slot] = gr;
    }
}

// Radiance of ended path `pid` (slot `slot`): into the sample buffer at its
// path index (the film kernel gathers it), or as its Li.
__device__ __forceinline__ void store_sample(const RenderParams& P, unsigned long long pid, float3 L, int slot) {
    if (!slot_ok(P, slot) || !DL_IN_BOUNDS(pid < P.cnt->pass_total, &P.cnt->err)) return;
    if (P.mode == 1) {
        P.li_L[3 * pid] = L.x;
        P.li_L[3 * pid + 1] = L.y;
        P.li_L[3 * pid + 2] = L.z;
        float2 ps = P.pos[slot];
        P.li_pos[2 * pid] = ps.x;
        P.li_pos[2 * pid + 1] = ps.y;
    } else {
        P.samples[pid] = make_float4(L.x, L.y, L.z, 1.f);
    }
}

// A shadow ray of an ended path was unoccluded: add its contribution to the
// stored sample.  One shadow ray per path at a time, so no atomics.
__device__ __forceinline__ void add_to_sample(const RenderParams& P, unsigned long long pid, float4 c) {
    if (!DL_IN_BOUNDS(pid < P.cnt->pass_total, &P.cnt->err)) return;
    if (P.mode == 1) {
        P.li_L[3 * pid] = __fadd_rn(P.li_L[3 * pid], c.x);
        P.li_L[3 * pid + 1] = __fadd_rn(P.li_L[3 * pid + 1], c.y);
        P.li_L[3 * pid + 2] = __fadd_rn(P.li_L[3 * pid + 2], c.z);
    } else {
        float4 s = P.samples[pid];
        P.samples[pid] = make_float4(__fadd_rn(s.x, c.x), __fadd_rn(s.y, c.y), __fadd_rn(s.z, c.z), s.w);
    }
}

// Radiance `c` reached the path: credit it to the training records of its
// guided vertices (the newer one too if `both`), divided by the throughput
// after each vertex (mean over the channels it is non-zero in).
__device__ __forceinline__ void credit_one(const RenderParams& P, float4 t, float3 c) {
    int idx = __float_as_int(t.w);
    if (idx < 0) return;
    float s = 0.f;
    int k = 0;
    if (t.x > 0.f) { s += c.x / t.x; k++; }
    if (t.y > 0.f) { s += c.y / t.y; k++; }
    if (t.z > 0.f) { s += c.z / t.z; k++; }
    if (k > 0 && isfinite(s)) static_cast<GuideRecord*>(P.cnt->pass_recs)[idx].L += s / (float)k;
}
__device__ __forceinline__ void credit(const RenderParams& P, const GuideRec& gr, float3 c, bool both) {
    credit_one(P, gr.a, c);
    if (both) credit_one(P, gr.b, c);
}

// Claim new path indices for the lanes in `want`, start them; returns true
// for lanes that now hold a fresh camera ray.
template <bool kMulti>
__device__ __forceinline__ bool regenerate(const RenderParams& P, int slot, bool want) {
    unsigned long long pid = warp_claim(&P.cnt->next_path, want);
    bool ok = want && pid < P.cnt->pass_total;
    if (ok) start_path<kMulti>(P, slot, pid);
    return ok;
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

// The emitter that the NEE sample's first number picks, that number rescaled
// to [0, 1) for reuse: uniformly (scene.cpp:148-163), or, with
// DL_RENDER_POWER_LIGHT_PICK, through the power alias table (slot from the
// number, alias coin from its fraction).
__device__ __forceinline__ int pick_light(const DevRequest& R, float& sx) {
    const DevScene& sc = R.sc;
    const int N = sc.num_lights;
    if (!(R.flags & DL_RENDER_POWER_LIGHT_PICK)) {
        if (N <= 1) return 0;
        int idx = min((int)__fmul_rn(sx, (float)N), N - 1);
        sx = __fsub_rn(__fmul_rn(sx, (float)N), (float)idx);
        return idx;
    }
    float u = __fmul_rn(sx, (float)N);
    int i = min((int)u, N - 1);
    float coin = fminf(__fsub_rn(u, (float)i), 0.99999994f);
    float4 a = __ldg(sc.light_pick + i);
    if (coin < a.x) {
        sx = __fdiv_rn(coin, a.x);
        return i;
    }
    sx = __fdiv_rn(__fsub_rn(coin, a.x), __fsub_rn(1.f, a.x));
    return __float_as_int(a.y);
}

// pdf of direction sample `pdf` of emitter `l` times its pick probability
// (pdfEmitterDirection, scene.cpp:171-179).
__device__ __forceinline__ float with_pick_pdf(const DevRequest& R, int l, float pdf) {
    if (R.flags & DL_RENDER_POWER_LIGHT_PICK) return __fmul_rn(pdf, __ldg(R.sc.light_pick + l).z);
    return R.sc.num_lights != 1 ? __fdiv_rn(pdf, (float)R.sc.num_lights) : pdf;
}

// Three fresh numbers for an envmap NEE sample, drawn after the NEE 2D sample.
__device__ __forceinline__ float3 env_xi(Pcg32& g) {
    float3 xi;
    xi.x = g.next_float();
    xi.y = g.next_float();
    xi.z = g.next_float();
    return xi;
}

// Scene::sampleEmitterDirection without the visibility test (the caller
// traces the shadow ray).  Returns the unoccluded spectrum.  An envmap pick
// draws three more numbers from `g`.
__device__ __forceinline__ float3 sample_emitter(const DevRequest& R, float3 its_p, float3 sh_n, float2 s,
                                                 Pcg32& g, float3& d, float& dist, float& pdf, bool& delta) {
    const DevScene& sc = R.sc;
    int N = sc.num_lights;
    float3 zero = f3(0.f, 0.f, 0.f);
    delta = false;
    pdf = 0.f;
    dist = 0.f;
    d = zero;
    if (N == 0) return zero;
    const int idx = pick_light(R, s.x);
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
        if (R.flags & DL_RENDER_FIX_POINT_LIGHT) {
            float c = fmaxf(dot(sh_n, d), 0.f);
            spec = c > 0.f ? scale(scale(scale(ld3(L.radiance), c), inv), inv) : zero;
        } else {
            spec = scale(scale(ld3(L.radiance), inv), inv);
        }
    } else if (L.type == LIGHT_ENVMAP) {
        spec = env_sample(sc, sh_n, env_xi(g), d, pdf);
        dist = 1e16f;  // envmap.h:67
    } else {
        spec = zero;
    }
    if (R.flags & DL_RENDER_POWER_LIGHT_PICK) {
        const float pl = __ldg(sc.light_pick + idx).z;
        spec = divs(spec, pl);
        pdf = __fmul_rn(pdf, pl);
    } else if (N > 1) {
        spec = scale(spec, (float)N);
        pdf = __fmul_rn(pdf, __fdiv_rn(1.f, (float)N));
    }
    return spec;
}

// ---------------------------------------------------------------- kernels
// First camera paths of a pass: slot i starts path i (no claiming needed),
// and the extension queue lists the started slots in order.
template <bool kMulti>
__global__ void k_init(RenderParams P, int capacity) {
    const unsigned long long total = P.cnt->pass_total;
    int n = (int)min((unsigned long long)capacity, total);
    if (!DL_IN_BOUNDS(capacity <= P.capacity, &P.cnt->err)) n = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        P.cnt->next_path = (unsigned long long)n;
        P.cnt->ext[0] = n;
    }
    for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < n; slot += gridDim.x * blockDim.x) {
        start_path<kMulti>(P, slot, (unsigned long long)slot);
        P.ext_q[0][slot] = slot;
    }
}

// traversal state: ray finished (below every leaf reference: scenes hold
// fewer than 2^27 triangles)
constexpr int kDone = INT_MIN;

// Persistent traversal over a ray queue.  Each lane holds one ray's
// traversal state (node, stack); a lane whose ray finishes takes the next ray
// of the queue, so lanes do not idle while the warp's longest ray finishes.
// A warp reserves queue entries kFetchChunk at a time (one atomic per chunk)
// and hands them to its lanes as they free up.
//   kAny = false: closest hit of extension rays E[p] (slots) -> hit[slot], and
//                 the slot joins the queue of its hit's material type (or the
//                 miss queue).  Each warp stages those entries per destination
//                 in shared memory and appends them 32 at a time: one atomic
//                 and one coalesced 128-byte store per 32 entries.
//   kAny = true:  any hit of shadow rays S (queue positions); unoccluded ones
//                 add their contribution to the path or the ended path's sample
constexpr unsigned kFetchChunk = 64;
constexpr int kTraverseWarps = 4;  // 128 threads
constexpr int kStage = 64;         // staged entries per warp and destination (flushed at 32)
constexpr int kSmemStack = 8;      // top traversal-stack entries per thread kept in shared memory

template <bool kCount, bool kAny, bool kMulti>
__global__ void __launch_bounds__(128) k_traverse(RenderParams P, int p) {
    const int q = p ^ 1;
    int n = kAny ? P.cnt->shadow[p] : P.cnt->ext[p];
    if (!DL_IN_BOUNDS(n >= 0 && n <= P.capacity, &P.cnt->err)) n = 0;
    unsigned int* work = kAny ? &P.cnt->work_sh : &P.cnt->work_ext;
    constexpr int kDests = kAny ? 1 : kNumMaterialTypes + 1;
    __shared__ int s_qbuf[kTraverseWarps][kDests][kStage];
    __shared__ int s_qcnt[kTraverseWarps][kDests];
    const int warp = threadIdx.x >> 5, lane = lane_id();
    const unsigned lt = (1u << lane) - 1u;
    if (lane < kDests) s_qcnt[warp][lane] = 0;
    __syncwarp();
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (!kAny) {
            // this iteration's output queues start empty
            P.cnt->ext[q] = 0;
            P.cnt->shadow[q] = 0;
            P.cnt->stat_ext += (unsigned long long)n;
        } else {
            // next iteration's material queues start empty (the extension
            // traversal, which may run concurrently, appends to mat[p])
            for (int k = 0; k <= kNumMaterialTypes; k++) P.cnt->mat[q][k].n = 0;
            P.cnt->stat_shadow += (unsigned long long)n;
        }
    }
    uint32_t err = 0, nn = 0, nt = 0;
    bool has = false, exhausted = false;
    int idx = 0, slot = 0, node = kDone, sp = 0, hit_tri = -1, hit_mat = 0;
    float3 o = f3(0.f, 0.f, 0.f), d = o;
    float tmin = 0.f, tmax = 0.f, ht = 0.f, hu = 0.f, hv = 0.f;
    RayBox rb;
    rb.idir = o;
    rb.ood = o;
    // traversal stack: the first kSmemStack entries in shared memory, laid out
    // [depth][thread] so that lanes at different depths hit different banks;
    // deeper entries in local memory
    __shared__ int s_stack[kSmemStack][kTraverseWarps * 32];
    int stack[kStackSize - kSmemStack];
    int* const my_stack = &s_stack[0][threadIdx.x];
    auto push = [&](int v) {
        if (sp < kSmemStack) my_stack[sp * kTraverseWarps * 32] = v;
        else stack[sp - kSmemStack] = v;
        sp++;
    };
    auto pop = [&]() -> int {
        --sp;
        return sp < kSmemStack ? my_stack[sp * kTraverseWarps * 32] : stack[sp - kSmemStack];
    };
    int rid = 0;  // the ray's request
    const float4* nodes = P.r0.sc.nodes;
    const float4* tris = P.r0.sc.tris;
    int ntris = P.r0.sc.num_tris;
    unsigned c_next = 0, c_end = 0;  // the warp's reserved queue entries [c_next, c_end)
    for (;;) {
        bool need = !has && !exhausted;
        unsigned m = __ballot_sync(0xffffffffu, need);
        if (m) {
            const unsigned k = __popc(m), rank = __popc(m & lt), avail = c_end - c_next;
            unsigned mine;
            if (k > avail) {  // warp-uniform: reserve the next chunk
                unsigned base = 0;
                if (lane == 0) base = atomicAdd(work, kFetchChunk);
                base = __shfl_sync(0xffffffffu, base, 0);
                mine = rank < avail ? c_next + rank : base + (rank - avail);
                c_next = base + (k - avail);
                c_end = base + kFetchChunk;
            } else {
                mine = c_next + rank;
                c_next += k;
            }
            if (need) {
                idx = (int)min(mine, (unsigned)n);
                if (mine < (unsigned)n) {
                    float4 ro = make_float4(0.f, 0.f, 0.f, 0.f), rd = make_float4(0.f, 0.f, 0.f, -1.f);
                    if (kAny) {
                        ro = P.sh_o[idx];
                        rd = P.sh_d[idx];
                    } else {
                        slot = P.ext_q[p][idx];
                        if (slot_ok(P, slot)) {
                            RayRec r = P.rec[slot].ray;
                            ro = r.o;
                            rd = r.d;
                        }
                    }
                    o = xyz(ro);
                    d = xyz(rd);
                    tmin = kRayEps;
                    tmax = rd.w;
                    if (kMulti) {
                        rid = __float_as_int(ro.w);
                        const DevScene& rs = P.reqs[rid].sc;
                        nodes = rs.nodes;
                        tris = rs.tris;
                        ntris = rs.num_tris;
                    }
                    rb = make_raybox(o, d);
                    node = ntris > 0 ? 0 : kDone;
                    sp = 0;
                    hit_tri = -1;
                    has = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, has) == 0) break;
        bool finished = false;
        int dest = 0;
        if (has) {
            // descend inner nodes until a leaf (or the end of the traversal)
            while (node >= 0) {
#ifdef DL_CHECKS
                const int num_nodes = kMulti ? P.reqs[rid].sc.num_nodes : P.r0.sc.num_nodes;
                if (!DL_IN_BOUNDS(node < num_nodes, &P.cnt->err)) {
                    node = kDone;
                    break;
                }
#endif
                const float4* np = nodes + 4 * node;
                float4 a, b, c, dd;
                ld_nc_256(np, a, b);        // a node is two 32-byte halves
                ld_nc_256(np + 2, c, dd);
                const int2 ch = make_int2(__float_as_int(dd.x), __float_as_int(dd.y));
                if (kCount) nn++;
                bool h0, h1;
                float t0, t1;
                box2(rb, tmin, tmax, a, b, c, h0, h1, t0, t1);
                if (h0 && h1) {   // (both slots always hold a child: see bvh.h)
                    int near = ch.x, far = ch.y;
                    if (t1 < t0) { near = ch.y; far = ch.x; }
#ifdef DL_CHECKS
                    if (sp < kStackSize) push(far); else err |= 1u;
#else
                    push(far);   // depth <= kStackSize + 1: checked when the scene is built
#endif
                    node = near;
                } else if (h0) {
                    node = ch.x;
                } else if (h1) {
                    node = ch.y;
                } else {
                    node = sp > 0 ? pop() : kDone;
                }
            }
            finished = node == kDone;
            if (!finished) {
                // leaf: test its triangles (the reference's Moller-Trumbore)
                int ref = ~node;
                int first = ref >> 4, count = (ref & 15) + 1;
                if (!DL_IN_BOUNDS(first >= 0 && first + count <= ntris, &P.cnt->err)) count = 0;
                bool any = false;
                for (int k = 0; k < count; k++) {
                    const float4* tp = tris + 3 * (first + k);
                    float4 p0 = __ldg(tp), p1 = __ldg(tp + 1), p2 = __ldg(tp + 2);
                    if (kCount) nt++;
                    float t, u, v;
                    if (intersect_tri(xyz(p0), xyz(p1), xyz(p2), o, d, tmin, tmax, t, u, v)) {
                        if (kAny) {
                            any = true;
                            break;
                        }
                        tmax = t;
                        ht = t;
                        hu = u;
                        hv = v;
                        hit_tri = first + k;
                        hit_mat = __float_as_int(p1.w);  // material type of the triangle's mesh
                    }
                }
                if (kAny && any) {
                    finished = true;
                    hit_tri = 0;
                } else {
                    node = sp > 0 ? pop() : kDone;
                    finished = node == kDone;
                }
            }
            if (finished) {
                if (kAny) {
                    if (hit_tri < 0) {  // unoccluded: add the NEE contribution
                        float4 c = P.sh_c[idx];
                        int target = __float_as_int(c.w);
                        if (target >= 0) {
                            if (slot_ok(P, target)) {
                                PathRec pr = P.rec[target].path;
                                pr.L = make_float4(__fadd_rn(pr.L.x, c.x), __fadd_rn(pr.L.y, c.y),
                                                   __fadd_rn(pr.L.z, c.z), pr.L.w);
                                P.rec[target].path = pr;
                                // NEE at the newest guided vertex feeds the record before it
                                if (P.guided) credit(P, P.grec[target], xyz(c), false);
                            }
                        } else {
                            add_to_sample(P, (unsigned long long)(unsigned)(-1 - target), c);
                        }
                    }
                } else {
                    HitRec hr;
                    hr.pad = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (hit_tri >= 0) {
                        hr.h = make_float4(ht, hu, hv, __int_as_float(hit_tri));
                        dest = hit_mat;
                    } else {
                        hr.h = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
                        dest = kMissQueue;
                    }
                    if (slot_ok(P, slot)) P.rec[slot].hit = hr;
                }
                has = false;
            }
        }
        if (!kAny) {
            unsigned fm = __ballot_sync(0xffffffffu, finished);
            while (fm) {  // warp-uniform loop over the destinations present
                const int dd = __shfl_sync(0xffffffffu, dest, __ffs(fm) - 1);
                const unsigned g = __ballot_sync(0xffffffffu, finished && dest == dd);
                fm &= ~g;
                int* buf = s_qbuf[warp][dd];
                int c = s_qcnt[warp][dd];
                if ((g >> lane) & 1u) buf[c + __popc(g & lt)] = slot;
                c += __popc(g);
                __syncwarp();
                if (c >= 32) {
                    int base = 0;
                    if (lane == 0) base = atomicAdd(&P.cnt->mat[p][dd].n, 32);
                    base = __shfl_sync(0xffffffffu, base, 0);
                    if (DL_IN_BOUNDS(base + 32 <= P.capacity, &P.cnt->err)) P.mat_q[dd][base + lane] = buf[lane];
                    const int rest = c - 32;
                    const int v = lane < rest ? buf[32 + lane] : 0;
                    __syncwarp();
                    if (lane < rest) buf[lane] = v;
                    c = rest;
                }
                __syncwarp();
                if (lane == 0) s_qcnt[warp][dd] = c;
                __syncwarp();
            }
        }
    }
    if (!kAny) {  // flush the staged remainders
        for (int dd = 0; dd < kDests; dd++) {
            const int c = s_qcnt[warp][dd];
            if (c == 0) continue;
            int base = 0;
            if (lane == 0) base = atomicAdd(&P.cnt->mat[p][dd].n, c);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (lane < c && DL_IN_BOUNDS(base + c <= P.capacity, &P.cnt->err))
                P.mat_q[dd][base + lane] = s_qbuf[warp][dd][lane];
        }
    }
    if (err) atomicOr(&P.cnt->err, err);
    if (kCount) {
        if (kAny) {
            atomicAdd(&P.cnt->stat_nodes_sh, (unsigned long long)nn);
            atomicAdd(&P.cnt->stat_tris_sh, (unsigned long long)nt);
        } else {
            atomicAdd(&P.cnt->stat_nodes_ext, (unsigned long long)nn);
            atomicAdd(&P.cnt->stat_tris_ext, (unsigned long long)nt);
        }
    }
}

// Rays that hit nothing (path.cpp:23-25, 85-87): with an envmap, add its
// radiance first (miss.cu:11-49: camera rays see it if "visual", else the
// background colour; later rays weight it by MIS against the BSDF pdf after
// a diffuse bounce).  Store the sample, then start new camera paths in the
// freed slots.
template <bool kMulti, int kThreads>
__global__ void __launch_bounds__(kThreads) k_miss(RenderParams P, int p) {
    const int q = p ^ 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) {  // next iteration's traversal cursors (both traversals are done)
        P.cnt->work_ext = 0;
        P.cnt->work_sh = 0;
    }
    int n = P.cnt->mat[p][kMissQueue].n;
    if (!DL_IN_BOUNDS(n >= 0 && n <= P.capacity, &P.cnt->err)) n = 0;
    // Every queued miss starts a new path in its slot.  A warp's entries over
    // the whole launch are known (i0 = w0 + j * stride, all lanes but the
    // last round's tail), so it claims their path indices, and queue
    // positions for the ones the pass still has, with one atomic each; the
    // started paths are a prefix of the warp's entries.
    const int stride = gridDim.x * blockDim.x;
    const int w0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31;
    int count = 0;
    for (int i0 = w0; i0 < n; i0 += stride) count += min(32, n - i0);
    const unsigned long long total = P.cnt->pass_total;
    unsigned long long pid0 = 0;
    int e0 = 0;
    if (lane_id() == 0 && count > 0) {
        pid0 = atomicAdd(&P.cnt->next_path, (unsigned long long)count);
        const int starts = pid0 < total ? (int)min((unsigned long long)count, total - pid0) : 0;
        if (starts > 0) e0 = atomicAdd(&P.cnt->ext[q], starts);
    }
    pid0 = __shfl_sync(0xffffffffu, pid0, 0);
    e0 = __shfl_sync(0xffffffffu, e0, 0);
    int done_before = 0;  // the warp's entries in earlier rounds
    for (int i0 = w0; i0 < n; i0 += stride) {
        int i = i0 + lane_id();
        bool active = i < n;
        int slot = active ? P.mat_q[kMissQueue][i] : 0;
        if (active && !slot_ok(P, slot)) active = false;
        if (active) {
            PathRec pr = P.rec[slot].path;
            int4 m = P.rec[slot].meta.m;
            const DevRequest& R = request<kMulti>(P, m.y >> kReqShift);
            const DevScene& sc = R.sc;
            float3 L = f3(pr.L.x, pr.L.y, pr.L.z);
            // (the normals integrator returns 0 on a miss, normal.cpp:13-14)
            if (sc.env_light >= 0 && !(R.flags & DL_RENDER_NORMALS)) {
                float3 dir = xyz(P.rec[slot].ray.d);
                if (m.y & PF_CAMERA) {
                    L = add(L, sc.env_visual ? env_lookup_dir(sc, dir) : ld3(sc.env_bg));
                } else {
                    float3 le = env_lookup_dir(sc, dir);
                    float w = 1.f;
                    if (m.y & PF_PREV_DIFFUSE) {
                        float ep = env_pdf(sc, dir);
                        ep = with_pick_pdf(R, sc.env_light, ep);
                        w = mis_weight(pr.L.w, ep);
                    }
                    float3 c = mul(scale(f3(pr.tp.x, pr.tp.y, pr.tp.z), w), le);
                    L = add(L, c);
                    if (P.guided) credit(P, P.grec[slot], c, true);
                }
            }
            store_sample(P, path_index(m), L, slot);
        }
        const int r = done_before + lane_id();
        const unsigned long long pid = pid0 + (unsigned long long)r;
        if (active && pid < total) {
            start_path<kMulti>(P, slot, pid);
            if (DL_IN_BOUNDS(e0 + r < P.capacity, &P.cnt->err)) P.ext_q[q][e0 + r] = slot;
        }
        done_before += min(32, n - i0);
    }
}

// One BSDF type, the whole rest of the path iteration for hits on it:
// emitter hit + MIS (path.cpp:72-84) or first-hit emission (27-29), Russian
// roulette (89-97), depth limit, next-event estimation (36-56) and BSDF
// sampling (60-69).  A path that ends here stores its sample and its slot
// starts a new camera path at once; a shadow ray it emitted on the way adds
// to the stored sample when traced.  Mirror and dielectric still draw the NEE
// sample (their eval and pdf are zero: no contribution, no shadow ray).
//
// kGuided (diffuse, Beckmann, GGX in a guided render): blocks of two
// warpgroups; each warpgroup takes 128 queued hits at a time and evaluates
// the guiding network for them on the tensor cores (guide_tc.cuh:
// tcgen05.mma, accumulators in tensor memory);
// each path samples its next direction by one-sample MIS between the learned
// vMF mixture (probability `fraction`) and the BSDF, weighting by
// f cos / (fraction q + (1 - fraction) p_bsdf); NEE's MIS weight uses the
// same combined pdf.  The vertex becomes a training record.
constexpr size_t kGuidedSmem = sizeof(GuideTcSmem);

template <int T, bool kMulti, bool kGuided, int kThreads>
__global__ void __launch_bounds__(kGuided ? kTcThreads : kThreads) k_material(RenderParams P, int p) {
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    const int q = p ^ 1;
    const int lane = lane_id();
    int n = P.cnt->mat[p][T].n;
    if (!DL_IN_BOUNDS(n >= 0 && n <= P.capacity, &P.cnt->err)) n = 0;
    // guided: each warpgroup walks whole 128-row tiles (every thread takes
    // part in the network's warpgroup-wide steps); otherwise each warp walks
    // 32 rows
    constexpr int kSpan = kGuided ? kTcRows : 32;
    // training-record bookkeeping: guided kernels, and mirror / dielectric
    // hits of a guided render (the other types then run their guided kernel)
    constexpr bool kMayGuide = kGuided || (!kMulti && (T == MAT_MIRROR || T == MAT_DIELECTRIC));
    const bool guided = kMayGuide && P.guided;
    uint32_t mma_phase = 0;
    bool net_ok = false;
    if (kGuided) {
        if ((int)blockIdx.x * kTcThreads >= n) return;
        net_ok = guide_tc_begin(*reinterpret_cast<GuideTcSmem*>(dyn_smem), P.gnet.image, &P.cnt->err);
    }
    for (int i0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~(kSpan - 1); i0 < n; i0 += gridDim.x * blockDim.x) {
        int i = i0 + (kGuided ? tc_row() : lane);
        bool active = i < n;
        int slot = active ? P.mat_q[T][i] : 0;
        if (active && !slot_ok(P, slot)) active = false;
        bool cont = false, emit = false, done = false;
        float4 sh_o = make_float4(0.f, 0.f, 0.f, 0.f), sh_d = sh_o, sh_c = sh_o;
        // ---- phase 1: emitter hit, Russian roulette, depth limit
        RayRec ray;
        PathRec pr;
        MetaRec mr;
        Pcg32 g;
        HitInfo h;
        GuideRec gr;
        float2 tuv = make_float2(0.f, 0.f);  // texture coordinates (textured materials)
        float3 s_tan = f3(0.f, 0.f, 0.f);    // aniso_ggx: shading tangent from a tangent map
        float3 tp = f3(0.f, 0.f, 0.f), Lr = tp, dir = tp;
        float eta = 1.f;
        int depth = 0, flags = 0, rid = 0;
        unsigned long long pid = 0;
        if (active) {
            float4 hit = P.rec[slot].hit.h;
            ray = P.rec[slot].ray;
            pr = P.rec[slot].path;
            mr = P.rec[slot].meta;
            if (guided) gr = P.grec[slot];
            g = load_rng(mr.rng);
            pid = path_index(mr.m);
            tp = f3(pr.tp.x, pr.tp.y, pr.tp.z);
            eta = pr.tp.w;
            Lr = f3(pr.L.x, pr.L.y, pr.L.z);
            dir = xyz(ray.d);
            depth = mr.m.x;
            flags = mr.m.y;
            rid = flags >> kReqShift;
            const DevRequest& R = request<kMulti>(P, rid);
            const DevScene& sc = R.sc;
            if (!DL_IN_BOUNDS(__float_as_int(hit.w) >= 0 && __float_as_int(hit.w) < sc.num_tris, &P.cnt->err))
                hit.w = __int_as_float(0);
            h = hit_info(sc, __float_as_int(hit.w), hit.y, hit.z);
            if (T == MAT_DIFFUSE || T == MAT_ANISO_GGX) {
                const DevMaterial& mt = sc.materials[sc.meshes[h.mesh].material];
                if (mt.has_tex) {
                    tuv = hit_texcoord(sc, __float_as_int(hit.w), hit.y, hit.z);
                    // world-space normal / tangent maps (shader_common.h:62-64,
                    // 104-107): normalize(2 rgb - 1) replaces the shading normal
                    if (T == MAT_ANISO_GGX && mt.tex[TEX_NORMAL] >= 0) {
                        const float3 c = tex_lookup(sc, mt.tex[TEX_NORMAL], tuv);
                        h.sh.n = normalize(f3(__fsub_rn(__fmul_rn(c.x, 2.f), 1.f), __fsub_rn(__fmul_rn(c.y, 2.f), 1.f),
                                              __fsub_rn(__fmul_rn(c.z, 2.f), 1.f)));
                    }
                    if (T == MAT_ANISO_GGX && mt.tex[TEX_TANGENT] >= 0) {
                        const float3 c = tex_lookup(sc, mt.tex[TEX_TANGENT], tuv);
                        s_tan = normalize(f3(__fsub_rn(__fmul_rn(c.x, 2.f), 1.f), __fsub_rn(__fmul_rn(c.y, 2.f), 1.f),
                                             __fsub_rn(__fmul_rn(c.z, 2.f), 1.f)));
                    }
                }
            }
            int light = sc.meshes[h.mesh].light;
            if (R.flags & DL_RENDER_NORMALS) {
                // the normals integrator (normal.cpp:10-20): |shading normal|
                // of the first hit, and the path ends
                Lr = f3(fabsf(h.sh.n.x), fabsf(h.sh.n.y), fabsf(h.sh.n.z));
                done = true;
            } else if (flags & PF_CAMERA) {
                if (light >= 0 && dot(h.sh.n, neg(dir)) > 0.f) Lr = add(Lr, mul(tp, ld3(sc.lights[light].radiance)));
                depth = 0;
            } else {
                if (light >= 0) {
                    const DevLight& Lt = sc.lights[light];
                    float3 le = dot(h.sh.n, neg(dir)) > 0.f ? ld3(Lt.radiance) : f3(0.f, 0.f, 0.f);
                    float3 vec = sub(h.p, xyz(ray.o));
                    float3 dd = normalize(vec);
                    float dist = length(vec);
                    float dp = fmaxf(dot(h.sh.n, neg(dd)), 0.f);
                    float ep = dp != 0.f ? __fdiv_rn(__fmul_rn(__fmul_rn(Lt.pA, dist), dist), dp) : 0.f;
                    ep = with_pick_pdf(R, light, ep);
                    float w = (flags & PF_PREV_DIFFUSE) ? mis_weight(pr.L.w, ep) : 1.f;
                    float3 c = mul(scale(tp, w), le);
                    Lr = add(Lr, c);
                    if (guided) credit(P, gr, c, true);
                }
                if (depth > R.rr_depth) {
                    float pq = fminf(maxc(scale(scale(tp, eta), eta)), 0.99f);
                    if (g.next_float() > pq) done = true;
                    else tp = divs(tp, pq);
                }
                depth += 1;
            }
            if (!done && R.max_depth > 0 && depth >= R.max_depth) done = true;
        }
        // ---- phase 2 (guided): the network on the block's 128 shading points
        const bool sampling = active && !done;
        bool use_guide = kGuided && sampling && depth < P.gnet.max_depth;
        float in6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        float* lob = nullptr;
        if (kGuided) {
            GuideTcSmem& S = *reinterpret_cast<GuideTcSmem*>(dyn_smem);
            const int grp = tc_group();
            lob = tc_out_row(S, grp, tc_row());
            if (use_guide) guide_input(request<kMulti>(P, rid).sc, h.p, normalize(h.sh.n), in6);
            // (also the barrier after which the previous tile's lobes are dead)
            if (wg_or(grp, use_guide) && net_ok) {
                encode_row_tc(in6, S.act[grp], tc_row());
                net_ok = guide_tc_forward(S, grp, mma_phase, &P.cnt->err);
            }
            if (!net_ok) use_guide = false;  // a wait ran out: sample the BSDF alone
            if (use_guide) decode_lobes_inplace(lob);
        }
        // ---- phase 3: NEE and the next direction
        bool record = false, rotate = false;
        float rec_pdf = 0.f;
        float3 nd = f3(0.f, 0.f, 0.f);
        if (active) {
            const DevRequest& R = request<kMulti>(P, rid);
            const DevScene& sc = R.sc;
            float prev_pdf = pr.L.w;
            int target = slot;
            if (!done) {
                DevMaterial m = sc.materials[sc.meshes[h.mesh].material];
                if ((T == MAT_DIFFUSE || T == MAT_ANISO_GGX) && m.has_tex) {
                    // texture lookups replace the constants (diffuse.cu:15-20,
                    // aniso_ggx.cu:19-35)
                    if (m.tex[TEX_ALBEDO] >= 0) {
                        const float3 a = tex_lookup(sc, m.tex[TEX_ALBEDO], tuv);
                        m.albedo[0] = a.x;
                        m.albedo[1] = a.y;
                        m.albedo[2] = a.z;
                    }
                    if (T == MAT_ANISO_GGX && m.tex[TEX_SPECULAR] >= 0) {
                        const float3 a = tex_lookup(sc, m.tex[TEX_SPECULAR], tuv);
                        m.specular[0] = a.x;
                        m.specular[1] = a.y;
                        m.specular[2] = a.z;
                    }
                    if (T == MAT_ANISO_GGX && m.tex[TEX_ALPHA] >= 0) {
                        const float3 a = tex_lookup(sc, m.tex[TEX_ALPHA], tuv);
                        m.ax = a.x;
                        m.ay = a.y;
                    }
                }
                Frame fr = T == MAT_ANISO_GGX ? make_onb_t(normalize(h.sh.n), s_tan) : h.sh;
                float3 wi = to_local(fr, neg(normalize(dir)));
                if (T == MAT_ANISO_GGX) wi = normalize(wi);
                const float alpha = use_guide ? P.gnet.fraction : 0.f;
                float2 s_nee = g.next2d();
                float3 c = f3(0.f, 0.f, 0.f);
                float3 ld = c;
                float ldist = 0.f;
                if (T == MAT_MIRROR || T == MAT_DIELECTRIC) {
                    // no NEE contribution, but an envmap pick still draws its numbers
                    float sx = s_nee.x;
                    if (sc.env_light >= 0 && sc.num_lights > 0 && pick_light(R, sx) == sc.env_light) (void)env_xi(g);
                } else {
                    float lpdf;
                    bool delta;
                    float3 espec = sample_emitter(R, h.p, h.sh.n, s_nee, g, ld, ldist, lpdf, delta);
                    if (__fadd_rn(__fadd_rn(espec.x, espec.y), espec.z) > 0.f && lpdf > 0.f) {
                        BRec q1;
                        q1.wi = wi;
                        q1.wo = to_local(fr, ld);
                        q1.measure = M_SOLID;
                        q1.eta = 1.f;
                        float3 bv = bsdf_eval<T>(m, q1);
                        float bp = bsdf_pdf<T>(m, q1);
                        if (use_guide) bp = alpha * stored_mixture_pdf(lob, ld) + (1.f - alpha) * bp;
                        float w = (delta && (R.flags & DL_RENDER_FIX_POINT_LIGHT)) ? 1.f : mis_weight(lpdf, bp);
                        c = mul(mul(scale(tp, w), bv), espec);
                        emit = c.x != 0.f || c.y != 0.f || c.z != 0.f;
                    }
                }
                BRec q2;
                q2.wi = wi;
                q2.wo = f3(0.f, 0.f, 0.f);
                q2.eta = 1.f;
                q2.measure = M_UNKNOWN;
                if (use_guide) {
                    // one-sample MIS between the learned mixture and the BSDF
                    float3 fcos_over_p;
                    if (g.next_float() < alpha) {
                        float u0 = g.next_float();
                        nd = stored_mixture_sample(lob, u0, g.next2d());
                        q2.wo = to_local(fr, nd);
                        q2.measure = M_SOLID;
                        float3 fv = bsdf_eval<T>(m, q2);
                        float pb = bsdf_pdf<T>(m, q2);
                        prev_pdf = alpha * stored_mixture_pdf(lob, nd) + (1.f - alpha) * pb;
                        fcos_over_p = prev_pdf > 0.f ? scale(fv, fmaxf(q2.wo.z, 0.f) / prev_pdf) : f3(0.f, 0.f, 0.f);
                    } else {
                        const float2 s2 = g.next2d();
                        const float lobe = T == MAT_ANISO_GGX ? g.next_float() : 0.f;
                        float3 wgt = bsdf_sample<T>(m, q2, s2, lobe);
                        float pb = bsdf_pdf<T>(m, q2);
                        nd = to_world(fr, q2.wo);
                        if (T == MAT_ANISO_GGX) nd = normalize(nd);
                        prev_pdf = alpha * stored_mixture_pdf(lob, nd) + (1.f - alpha) * pb;
                        fcos_over_p = prev_pdf > 0.f ? scale(wgt, pb / prev_pdf) : f3(0.f, 0.f, 0.f);
                    }
                    tp = mul(tp, fcos_over_p);
                    rec_pdf = prev_pdf;
                } else {
                    const float2 s2 = g.next2d();
                    const float lobe = T == MAT_ANISO_GGX ? g.next_float() : 0.f;
                    float3 f = bsdf_sample<T>(m, q2, s2, lobe);
                    tp = mul(tp, f);
                    eta = __fmul_rn(eta, q2.eta);
                    prev_pdf = bsdf_pdf<T>(m, q2);
                    nd = to_world(fr, q2.wo);
                    if (T == MAT_ANISO_GGX) nd = normalize(nd);
                }
                flags = (rid << kReqShift) | (is_diffuse(T) ? PF_PREV_DIFFUSE : 0);
                if (tp.x == 0.f && tp.y == 0.f && tp.z == 0.f) {
                    done = true;  // every later contribution is zero
                } else {
                    RayRec nr;
                    nr.o = make_float4(h.p.x, h.p.y, h.p.z, __int_as_float(rid));
                    nr.d = make_float4(nd.x, nd.y, nd.z, __int_as_float(0x7f800000));
                    P.rec[slot].ray = nr;
                    cont = true;
                    rotate = use_guide && P.grecords != nullptr;
                    record = rotate && (uint32_t)(splitmix64(pid * 64ull + (unsigned long long)depth) >> 40) <
                                           P.cnt->pass_keep;
                }
                if (emit) {
                    if (done) target = -1 - (int)pid;  // lands in the stored sample
                    sh_o = make_float4(h.p.x, h.p.y, h.p.z, __int_as_float(rid));
                    sh_d = make_float4(ld.x, ld.y, ld.z, __fsub_rn(ldist, kRayEps));
                    sh_c = make_float4(c.x, c.y, c.z, __int_as_float(target));
                }
            }
            if (done) {
                store_sample(P, pid, Lr, slot);
            } else {
                PathRec npr;
                npr.tp = make_float4(tp.x, tp.y, tp.z, eta);
                npr.L = make_float4(Lr.x, Lr.y, Lr.z, prev_pdf);
                P.rec[slot].path = npr;
                MetaRec nmr;
                nmr.m = make_int4(depth, flags, mr.m.z, mr.m.w);
                nmr.rng = store_rng(g);
                P.rec[slot].meta = nmr;
            }
        }
        // ---- phase 4 (guided): training record of the vertex (a hashed
        // subset of the guided vertices, spread over the whole pass)
        if (kGuided) {
            unsigned long long ri = warp_claim_u32(&P.cnt->guide_next, record);
            if (rotate) {
                int idx = record && ri < (unsigned long long)P.grecord_cap ? (int)ri : -1;
                if (idx >= 0) {
                    GuideRecord rc;
                    for (int k = 0; k < 6; k++) rc.in[k] = in6[k];
                    rc.w[0] = nd.x;
                    rc.w[1] = nd.y;
                    rc.w[2] = nd.z;
                    rc.pdf = rec_pdf;
                    rc.L = 0.f;
                    rc.pad = 0.f;
                    static_cast<GuideRecord*>(P.cnt->pass_recs)[idx] = rc;
                }
                GuideRec ngr;
                ngr.a = gr.b;
                ngr.b = make_float4(tp.x, tp.y, tp.z, __int_as_float(idx));
                P.grec[slot] = ngr;
            }
        }
        int sp = warp_push(&P.cnt->shadow[q], emit);
        if (emit && DL_IN_BOUNDS(sp < P.capacity, &P.cnt->err)) {
            P.sh_o[sp] = sh_o;
            P.sh_d[sp] = sh_d;
            P.sh_c[sp] = sh_c;
        }
        bool fresh = regenerate<kMulti>(P, slot, done);
        bool push = cont || fresh;
        int e = warp_push(&P.cnt->ext[q], push);
        if (push && DL_IN_BOUNDS(e < P.capacity, &P.cnt->err)) P.ext_q[q][e] = slot;
    }
    if (kGuided) guide_tc_end(*reinterpret_cast<GuideTcSmem*>(dyn_smem), mma_phase);
}

// Film accumulation as a gather (the reference splats each sample with
// ImageBlock::put, src/core/bitmap/block.cpp:81-113).  One block owns a
// 32x32 tile of film pixels; per sample index it stages the samples of the
// 36x36 image pixels around it (radiance from the sample buffer, film
// position recomputed from the path's pcg32 stream: its first 2D draw) in
// shared memory together with their 5 x and 5 y filter weights (the
// reference's table lookup).  Each thread then owns four film pixels of one
// column and sums the weighted samples of their 5x5 neighbourhoods; a staged
// sample's radiance and x weight are read once for all four.  Every pixel
// sums in a fixed order (sample index, then row, then column): no atomics,
// bit-reproducible films.  Samples the film rejects (NaN, Inf or negative:
// ImageBlock::put block.cpp:82-88) get zero weight and are counted.
constexpr int kFilmTile = 32, kFilmApron = 2, kFilmRegion = kFilmTile + 2 * kFilmApron, kFilmRows = 4;
constexpr int kFilmCells = kFilmRegion * kFilmRegion;
constexpr int kFilmTaps = 2 * kFilmApron + 1;  // 5 film pixels per axis around a sample
constexpr int kFilmThreads = kFilmTile * kFilmTile / kFilmRows;
// staged per cell: r, g, b, 5 x weights, 5 y weights
constexpr size_t kFilmSmem = (size_t)(3 + 2 * kFilmTaps) * kFilmCells * sizeof(float);

struct FilmParams {
    float4* film;
    const float4* samples;
    unsigned long long* invalid;
    int w, h, cols, rows, border;
    float lookup;
    float table[33];
    int nspp;             // samples per pixel in the sample buffer
    int s_first;          // sample index of the buffer's first sample
    unsigned long long seed_mix;
    int accumulate;       // add to the film instead of overwriting it
};

__global__ void __launch_bounds__(kFilmThreads) k_film_gather(FilmParams F) {
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    float* const s_r = reinterpret_cast<float*>(dyn_smem);
    float* const s_g = s_r + kFilmCells;
    float* const s_b = s_g + kFilmCells;
    float* const s_wx = s_b + kFilmCells;               // [kFilmTaps][kFilmCells]
    float* const s_wy = s_wx + kFilmTaps * kFilmCells;  // [kFilmTaps][kFilmCells]
    __shared__ float s_table[33];
    __shared__ unsigned int s_invalid;
    const int tx = threadIdx.x % kFilmTile, ty = threadIdx.x / kFilmTile;  // column, group of 4 rows
    const int X0 = blockIdx.x * kFilmTile, Y0 = blockIdx.y * kFilmTile;
    const int X = X0 + tx, Yb = Y0 + kFilmRows * ty;
    const int IX0 = X0 - F.border - kFilmApron, IY0 = Y0 - F.border - kFilmApron;
    const size_t npix = (size_t)F.w * F.h;
    if (threadIdx.x < 33) s_table[threadIdx.x] = F.table[threadIdx.x];
    if (threadIdx.x == 0) s_invalid = 0;
    __syncthreads();
    float ar[kFilmRows], ag[kFilmRows], ab[kFilmRows], aw[kFilmRows];
#pragma unroll
    for (int j = 0; j < kFilmRows; j++) ar[j] = ag[j] = ab[j] = aw[j] = 0.f;
    for (int k = 0; k < F.nspp; k++) {
        for (int e = threadIdx.x; e < kFilmCells; e += kFilmThreads) {
            const int rx = e % kFilmRegion, ry = e / kFilmRegion;
            const int sx = IX0 + rx, sy = IY0 + ry;
            float L0 = 0.f, L1 = 0.f, L2 = 0.f;
            bool ok = false;
            float px = 0.f, py = 0.f;
            if (sx >= 0 && sx < F.w && sy >= 0 && sy < F.h) {
                float4 L = F.samples[(size_t)k * npix + (size_t)sy * F.w + sx];
                ok = L.w != 0.f && L.x >= 0.f && L.y >= 0.f && L.z >= 0.f && isfinite(L.x) && isfinite(L.y) &&
                     isfinite(L.z);
                // each sample is counted by the tile that owns its pixel
                if (!ok && L.w != 0.f && rx >= kFilmApron && rx < kFilmApron + kFilmTile && ry >= kFilmApron &&
                    ry < kFilmApron + kFilmTile)
                    atomicAdd(&s_invalid, 1u);
                if (ok) {
                    Pcg32 g;
                    seed_path(g, F.seed_mix, F.w, F.h, sx, sy, F.s_first + k);
                    float2 ps = g.next2d();
                    float fx = __fadd_rn((float)sx, ps.x), fy = __fadd_rn((float)sy, ps.y);
                    px = __fsub_rn(__fsub_rn(fx, 0.5f), (float)(-F.border));
                    py = __fsub_rn(__fsub_rn(fy, 0.5f), (float)(-F.border));
                    L0 = L.x;
                    L1 = L.y;
                    L2 = L.z;
                }
            }
            s_r[e] = L0;
            s_g[e] = L1;
            s_b[e] = L2;
            // weights of this sample for film columns X0 + rx - d and rows Y0 + ry - d
#pragma unroll
            for (int d = 0; d < kFilmTaps; d++) {
                int cx = X0 + rx - d, cy = Y0 + ry - d;
                float wx = 0.f, wy = 0.f;
                if (ok && cx >= 0 && cx < F.cols)
                    wx = s_table[min((int)__fmul_rn(fabsf(__fsub_rn((float)cx, px)), F.lookup), 32)];
                if (ok && cy >= 0 && cy < F.rows)
                    wy = s_table[min((int)__fmul_rn(fabsf(__fsub_rn((float)cy, py)), F.lookup), 32)];
                s_wx[d * kFilmCells + e] = wx;
                s_wy[d * kFilmCells + e] = wy;
            }
        }
        __syncthreads();
        // region rows kFilmRows*ty + r reach this thread's pixel j when
        // dy = r - j is a filter tap; per pixel the order is dy, then dx
#pragma unroll
        for (int r = 0; r < kFilmRows + kFilmTaps - 1; r++) {
#pragma unroll
            for (int dx = 0; dx < kFilmTaps; dx++) {
                const int c = (kFilmRows * ty + r) * kFilmRegion + tx + dx;
                const float wx = s_wx[dx * kFilmCells + c];
                const float R = __fmul_rn(s_r[c], wx), G = __fmul_rn(s_g[c], wx), B = __fmul_rn(s_b[c], wx);
#pragma unroll
                for (int j = 0; j < kFilmRows; j++) {
                    const int dy = r - j;
                    if (dy < 0 || dy >= kFilmTaps) continue;
                    const float wy = s_wy[dy * kFilmCells + c];
                    ar[j] = __fmaf_rn(R, wy, ar[j]);
                    ag[j] = __fmaf_rn(G, wy, ag[j]);
                    ab[j] = __fmaf_rn(B, wy, ab[j]);
                    aw[j] = __fmaf_rn(wx, wy, aw[j]);
                }
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && s_invalid) atomicAdd(F.invalid, (unsigned long long)s_invalid);
    if (X >= F.cols) return;
#pragma unroll
    for (int j = 0; j < kFilmRows; j++) {
        const int Y = Yb + j;
        if (Y >= F.rows) break;
        float4* o = F.film + (size_t)Y * F.cols + X;
        if (F.accumulate) {
            float4 c = *o;
            *o = make_float4(__fadd_rn(c.x, ar[j]), __fadd_rn(c.y, ag[j]), __fadd_rn(c.z, ab[j]),
                             __fadd_rn(c.w, aw[j]));
        } else {
            *o = make_float4(ar[j], ag[j], ab[j], aw[j]);
        }
    }
}

// Per device, once per context: kernels whose shared memory exceeds the
// default 48 KB limit.
void render_setup_device() {
    DL_CUDA(cudaFuncSetAttribute(k_film_gather, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFilmSmem));
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
    rec.ensure(128 * c);
    pos.ensure(8 * c);
    for (DevBuf* b : {&sh_o, &sh_d, &sh_c}) b->ensure(16 * c);
    for (DevBuf* b : {&ext_q[0], &ext_q[1]}) b->ensure(4 * c);
    for (int k = 0; k <= kNumMaterialTypes; k++) mat_q[k].ensure(4 * c);
    counters.ensure(sizeof(RenderCounters));
    invalid.ensure(sizeof(unsigned long long));
    host_counters.ensure(sizeof(RenderCounters) + sizeof(unsigned long long));
    capacity = cap;
}

size_t RenderBuffers::device_bytes() const {
    size_t s = rec.bytes + pos.bytes + ext_q[0].bytes + ext_q[1].bytes +
               sh_o.bytes + sh_d.bytes + sh_c.bytes + counters.bytes + film.bytes + rgb.bytes + samples.bytes;
    for (int k = 0; k <= kNumMaterialTypes; k++) s += mat_q[k].bytes;
    return s;
}

constexpr int kKernelsPerIteration = 8;

// The material kernel of type T: guided (the network's tiles and weights in
// dynamic shared memory, as many blocks as fit at once) for the non-delta
// BSDFs of a guided render.
template <int T, bool kMulti>
static void launch_material(const RenderParams& P, int p, cudaStream_t st, int wb, int th) {
    constexpr bool kCanGuide = !kMulti && T != MAT_MIRROR && T != MAT_DIELECTRIC;
    if (kCanGuide && P.guided)
        k_material<T, false, true, kTcThreads><<<P.gnet.blocks, kTcThreads, kGuidedSmem, st>>>(P, p);
    else if (th > 128)  // compiled for 256-thread blocks
        k_material<T, kMulti, false, 256><<<wb, th, 0, st>>>(P, p);
    else
        k_material<T, kMulti, false, 128><<<wb, th, 0, st>>>(P, p);
}

template <bool kMulti>
static void launch_miss(const RenderParams& P, int p, cudaStream_t st, int wb, int th) {
    if (th > 128)
        k_miss<kMulti, 256><<<wb, th, 0, st>>>(P, p);
    else
        k_miss<kMulti, 128><<<wb, th, 0, st>>>(P, p);
}

// Launches one wavefront iteration (8 kernels) with the context's launch
// shape.  `ev`, when given, holds 8 events bracketing extend, shadow, the
// material kernels, miss (kernels then run one after another).  Otherwise,
// with `fj` given, independent kernels run concurrently on the context's
// side streams: the extension traversal (this iteration's rays: reads their
// ray records, writes hit records) beside the shadow traversal (the previous
// iteration's NEE rays: adds to path records), then the miss kernel beside
// the five material kernels (disjoint slots and queues), joined before the
// next iteration.
template <bool kMulti>
static void launch_iteration(const RenderParams& P, int p, cudaStream_t st, int sms, const TuneParams& tp,
                             bool count, cudaEvent_t* ev, const dl_context* fj) {
    const int tb = sms * tp.trav_ctas_per_sm, wb = sms * tp.shade_ctas_per_sm, th = 128, sth = tp.shade_threads;
    if (!ev && fj) {
        cudaEventRecord(fj->fork_ev, st);
        cudaStreamWaitEvent(fj->aux[0], fj->fork_ev, 0);
        if (count) {
            k_traverse<true, false, kMulti><<<tb, th, 0, st>>>(P, p);
            k_traverse<true, true, kMulti><<<tb, th, 0, fj->aux[0]>>>(P, p);
        } else {
            k_traverse<false, false, kMulti><<<tb, th, 0, st>>>(P, p);
            k_traverse<false, true, kMulti><<<tb, th, 0, fj->aux[0]>>>(P, p);
        }
        cudaEventRecord(fj->join_ev[0], fj->aux[0]);
        cudaStreamWaitEvent(st, fj->join_ev[0], 0);
    } else {
        if (ev) cudaEventRecord(ev[0], st);
        if (count) k_traverse<true, false, kMulti><<<tb, th, 0, st>>>(P, p);
        else k_traverse<false, false, kMulti><<<tb, th, 0, st>>>(P, p);
        if (ev) { cudaEventRecord(ev[1], st); cudaEventRecord(ev[2], st); }
        if (count) k_traverse<true, true, kMulti><<<tb, th, 0, st>>>(P, p);
        else k_traverse<false, true, kMulti><<<tb, th, 0, st>>>(P, p);
        if (ev) { cudaEventRecord(ev[3], st); cudaEventRecord(ev[4], st); }
    }
    if (!ev && fj) {
        cudaEventRecord(fj->fork_ev, st);
        for (int i = 0; i < dl_context::kAux; i++) cudaStreamWaitEvent(fj->aux[i], fj->fork_ev, 0);
        launch_miss<kMulti>(P, p, st, wb, sth);
        launch_material<MAT_DIFFUSE, kMulti>(P, p, fj->aux[0], wb, sth);
        launch_material<MAT_MIRROR, kMulti>(P, p, fj->aux[1], wb, sth);
        launch_material<MAT_DIELECTRIC, kMulti>(P, p, fj->aux[2], wb, sth);
        launch_material<MAT_MICROFACET, kMulti>(P, p, fj->aux[3], wb, sth);
        launch_material<MAT_ANISO_GGX, kMulti>(P, p, fj->aux[4], wb, sth);
        for (int i = 0; i < dl_context::kAux; i++) {
            cudaEventRecord(fj->join_ev[i], fj->aux[i]);
            cudaStreamWaitEvent(st, fj->join_ev[i], 0);
        }
    } else {
        launch_material<MAT_DIFFUSE, kMulti>(P, p, st, wb, sth);
        launch_material<MAT_MIRROR, kMulti>(P, p, st, wb, sth);
        launch_material<MAT_DIELECTRIC, kMulti>(P, p, st, wb, sth);
        launch_material<MAT_MICROFACET, kMulti>(P, p, st, wb, sth);
        launch_material<MAT_ANISO_GGX, kMulti>(P, p, st, wb, sth);
        if (ev) { cudaEventRecord(ev[5], st); cudaEventRecord(ev[6], st); }
        launch_miss<kMulti>(P, p, st, wb, sth);
    }
    if (ev) cudaEventRecord(ev[7], st);
}

static void bind_pool(RenderParams& P, const RenderBuffers& B) {
    P.capacity = (int)B.capacity;
    P.rec = B.rec.as<SlotRec>();
    P.pos = B.pos.as<float2>();
    P.ext_q[0] = B.ext_q[0].as<int>();
    P.ext_q[1] = B.ext_q[1].as<int>();
    for (int k = 0; k <= kNumMaterialTypes; k++) P.mat_q[k] = B.mat_q[k].as<int>();
    P.sh_o = B.sh_o.as<float4>();
    P.sh_d = B.sh_d.as<float4>();
    P.sh_c = B.sh_c.as<float4>();
    P.cnt = B.counters.as<RenderCounters>();
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

static DevRequest make_request(dl_scene* S, const dl_render_opts& o) {
    DevRequest R;
    std::memset(&R, 0, sizeof(R));
    R.sc = S->dev;
    R.pid_first = 0;
    R.spp_offset = o.spp_offset;
    R.max_depth = o.max_depth;
    R.rr_depth = o.rr_depth;
    R.flags = o.flags;
    R.seed_mix = splitmix64(o.seed);
    return R;
}

// The values that change from pass to pass live in the device counters (set
// after their reset), not in the kernel parameters: one captured graph serves
// every pass and frame.
struct PassValues {
    unsigned long long total;
    int spp_offset;
    unsigned keep;
    void* recs;
};
static_assert(sizeof(PassValues) == 24, "pass values layout");

// Wavefront loop over the paths [0, total) of one pass, until every path and
// every shadow ray has finished.  Adds the pass's counters into `acc` and
// per-kernel times into kms.  `multi`: paths of a request table.
static void run_wavefront(dl_context* ctx, RenderParams& P, int64_t cap, bool multi, bool count_traversal,
                          double* kms, int64_t& launches, int64_t& iters, RenderCounters& acc,
                          unsigned long long total, int spp_offset, unsigned keep, void* recs = nullptr) {
    cudaStream_t st = ctx->stream;
    RenderBuffers& B = ctx->render;
    const TuneParams tp = ctx->tune;
    const int batch = tp.iters_per_graph;
    DL_CUDA(cudaMemsetAsync(P.cnt, 0, sizeof(RenderCounters), st));
    B.host_pass.ensure(sizeof(PassValues));
    PassValues* pv = B.host_pass.as<PassValues>();
    pv->total = total;
    pv->spp_offset = spp_offset;
    pv->keep = keep;
    pv->recs = recs;
    DL_CUDA(cudaMemcpyAsync(&P.cnt->pass_total, pv, sizeof(PassValues), cudaMemcpyHostToDevice, st));
    const int sms = ctx->num_sms > 0 ? ctx->num_sms : 152;
    const bool timing = ctx->kernel_timing;
    const bool use_graph = !timing && !count_traversal;
    if (timing && (int)ctx->timing_events.size() < 8 * batch) {
        size_t have = ctx->timing_events.size();
        ctx->timing_events.resize(8 * batch);
        for (size_t k = have; k < ctx->timing_events.size(); k++) DL_CUDA(cudaEventCreate(&ctx->timing_events[k]));
    }
    auto iteration = [&](int k, bool count, cudaEvent_t* ev) {
        if (multi) launch_iteration<true>(P, k & 1, st, sms, tp, count, ev, ctx);
        else launch_iteration<false>(P, k & 1, st, sms, tp, count, ev, ctx);
    };
    if (use_graph) {
        std::vector<unsigned char> key(sizeof(P) + sizeof(int) + sizeof(cudaStream_t) + sizeof(TuneParams) + 1);
        unsigned char* kp = key.data();
        std::memcpy(kp, &P, sizeof(P));
        kp += sizeof(P);
        std::memcpy(kp, &sms, sizeof(int));
        kp += sizeof(int);
        std::memcpy(kp, &st, sizeof(cudaStream_t));
        kp += sizeof(cudaStream_t);
        std::memcpy(kp, &tp, sizeof(TuneParams));
        kp += sizeof(TuneParams);
        *kp = multi ? 1 : 0;
        if (!ctx->graph_exec || key != ctx->graph_key) {
            if (ctx->graph_exec) {
                cudaGraphExecDestroy(ctx->graph_exec);
                ctx->graph_exec = nullptr;
            }
            cudaGraph_t g = nullptr;
            DL_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            for (int k = 0; k < batch; k++) iteration(k, false, nullptr);
            DL_CUDA(cudaStreamEndCapture(st, &g));
            cudaError_t e = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                ctx->graph_exec = nullptr;
                throw Error(DL_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
            }
            ctx->graph_key = key;
        }
    }
    if (multi) k_init<true><<<sms * 16, 128, 0, st>>>(P, (int)cap);
    else k_init<false><<<sms * 16, 128, 0, st>>>(P, (int)cap);
    launches += 1;
    RenderCounters* hc = B.host_counters.as<RenderCounters>();
    for (;;) {
        if (use_graph) {
            DL_CUDA(cudaGraphLaunch(ctx->graph_exec, st));
        } else {
            for (int k = 0; k < batch; k++)
                iteration(k, count_traversal, timing ? &ctx->timing_events[8 * k] : nullptr);
        }
        iters += batch;
        launches += batch * kKernelsPerIteration;
        DL_CUDA(cudaGetLastError());
        DL_CUDA(cudaMemcpyAsync(hc, P.cnt, sizeof(RenderCounters), cudaMemcpyDeviceToHost, st));
        DL_CUDA(cudaStreamSynchronize(st));
        if (timing) {
            for (int k = 0; k < batch; k++)
                for (int j = 0; j < 4; j++) {
                    float ms = 0.f;
                    DL_CUDA(cudaEventElapsedTime(&ms, ctx->timing_events[8 * k + 2 * j],
                                                 ctx->timing_events[8 * k + 2 * j + 1]));
                    kms[j] += ms;
                }
        }
        if (hc->err & kErrBounds) throw Error(DL_ERR_QUEUE_OVERFLOW, kBoundsMessage);
        if (hc->err & kErrTensorWait) throw Error(DL_ERR_TIMEOUT, "tensor-core wait timed out in a guided kernel");
        if (hc->err) throw Error(DL_ERR_QUEUE_OVERFLOW, "traversal stack overflow");
        if (hc->ext[0] == 0 && hc->shadow[0] == 0 && hc->next_path >= total) break;
        if (iters > 1000000) throw Error(DL_ERR_TIMEOUT, "render did not converge");
    }
    acc.stat_camera += std::min<unsigned long long>(hc->next_path, total);
    acc.stat_ext += hc->stat_ext;
    acc.stat_shadow += hc->stat_shadow;
    acc.stat_nodes_ext += hc->stat_nodes_ext;
    acc.stat_tris_ext += hc->stat_tris_ext;
    acc.stat_nodes_sh += hc->stat_nodes_sh;
    acc.stat_tris_sh += hc->stat_tris_sh;
}

// Budget of the per-path sample buffer; larger frames render in passes of
// whole samples per pixel.
constexpr size_t kSampleBufferBytes = (size_t)4 << 30;

static FilmParams film_params(const DevCamera& cam, const DevRequest& R, int filter, float* d_film,
                              const float4* samples, unsigned long long* invalid) {
    FilmParams F;
    std::memset(&F, 0, sizeof(F));
    float radius;
    filter_setup(filter, radius, F.border, F.lookup, F.table);
    F.film = reinterpret_cast<float4*>(d_film);
    F.samples = samples;
    F.invalid = invalid;
    F.w = cam.w;
    F.h = cam.h;
    F.cols = cam.w + 2 * F.border;
    F.rows = cam.h + 2 * F.border;
    F.seed_mix = R.seed_mix;
    return F;
}

static void finish_stats(dl_context* ctx, const RenderCounters& acc, unsigned long long invalid, int64_t iters,
                         int64_t launches, const double* kms) {
    cudaStream_t st = ctx->stream;
    DL_CUDA(cudaEventRecord(ctx->ev1, st));
    DL_CUDA(cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    DL_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->stats.camera_rays = (int64_t)acc.stat_camera;
    ctx->stats.extension_rays = (int64_t)acc.stat_ext;
    ctx->stats.shadow_rays = (int64_t)acc.stat_shadow;
    ctx->stats.invalid_samples = (int64_t)invalid;
    ctx->stats.iterations = iters;
    ctx->stats.render_ms = ms;
    ctx->stats.extend_ms = kms[0];
    ctx->stats.shadow_ms = kms[1];
    ctx->stats.shade_ms = kms[2];
    ctx->stats.retire_ms = kms[3];
    ctx->stats.kernel_launches = launches;
}

static int64_t pool_capacity(dl_context* ctx, int64_t requested, unsigned long long paths) {
    int64_t cap = requested > 0 ? requested : ctx->tune.paths_in_flight;
    cap = std::min<int64_t>(cap, (int64_t)std::max<unsigned long long>(paths, 1ull));
    return ((cap + 31) / 32) * 32;
}

// Runs one render.  mode 0: the film (d_film) receives every sample through
// the gather kernel; mode 1: Li of li_n explicit paths (d_xys -> d_L, d_pos).
void render_run(dl_scene* S, const dl_render_opts& o, float* d_film, int64_t li_n, const int* d_xys,
                float* d_L, float* d_pos, bool count_traversal, RenderCounters* out_counters) {
    dl_context* ctx = S->ctx;
    cudaStream_t st = ctx->stream;
    const DevCamera& cam = S->dev.cam;
    RenderParams P;
    std::memset(&P, 0, sizeof(P));
    P.r0 = make_request(S, o);
    P.mode = li_n > 0 ? 1 : 0;
    const unsigned long long npix = (unsigned long long)cam.w * cam.h;
    const int spp = std::max(o.spp, 1);
    int chunk_spp = P.mode == 1 ? 1 : (int)std::max<size_t>(1, std::min<size_t>(spp, kSampleBufferBytes / (npix * 16)));
    unsigned long long chunk_total = P.mode == 1 ? (unsigned long long)li_n : npix * (unsigned long long)chunk_spp;
    const int64_t cap = pool_capacity(ctx, o.max_paths_in_flight, chunk_total);
    RenderBuffers& B = ctx->render;
    B.ensure(cap);
    bind_pool(P, B);
    P.xys = d_xys;
    P.li_L = d_L;
    P.li_pos = d_pos;
    if (P.mode == 0) {
        B.samples.ensure((size_t)chunk_total * 16);
        P.samples = B.samples.as<float4>();
    }
    double kms[4] = {0, 0, 0, 0};
    int64_t launches = 0, iters = 0;
    RenderCounters acc;
    std::memset(&acc, 0, sizeof(acc));
    DL_CUDA(cudaEventRecord(ctx->ev0, st));
    unsigned long long invalid = 0;
    if (P.mode == 1) {
        run_wavefront(ctx, P, cap, false, count_traversal, kms, launches, iters, acc, (unsigned long long)li_n, 0,
                      1u << 24);
    } else {
        FilmParams F = film_params(cam, P.r0, o.filter, d_film, P.samples, B.invalid.as<unsigned long long>());
        DL_CUDA(cudaMemsetAsync(F.invalid, 0, sizeof(unsigned long long), st));
        dim3 fgrid((F.cols + kFilmTile - 1) / kFilmTile, (F.rows + kFilmTile - 1) / kFilmTile);
        for (int s0 = 0; s0 < spp; s0 += chunk_spp) {
            int ns = std::min(chunk_spp, spp - s0);
            run_wavefront(ctx, P, cap, false, count_traversal, kms, launches, iters, acc,
                          npix * (unsigned long long)ns, o.spp_offset + s0, 1u << 24);
            F.nspp = ns;
            F.s_first = o.spp_offset + s0;
            F.accumulate = s0 > 0;
            k_film_gather<<<fgrid, kFilmThreads, kFilmSmem, st>>>(F);
            launches += 1;
            DL_CUDA(cudaGetLastError());
        }
        unsigned long long* hinv =
            reinterpret_cast<unsigned long long*>(B.host_counters.as<char>() + sizeof(RenderCounters));
        DL_CUDA(cudaMemcpyAsync(hinv, F.invalid, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        DL_CUDA(cudaStreamSynchronize(st));
        invalid = *hinv;
    }
    acc.stat_invalid = invalid;
    finish_stats(ctx, acc, invalid, iters, launches, kms);
    if (out_counters) *out_counters = acc;
}

// Guided progressive render: passes of 1, 1, 2, 4, ... samples per pixel
// (the last takes the rest).  During a pass every guided vertex writes a
// training record; after the pass (train) the records feed steps_per_pass
// Adam steps on consecutive batches, and the next pass samples with the
// updated network.  All passes add to one film: each sample is an unbiased
// estimate whichever network drew it.
// Blocks of a guided material launch: as many as are resident at once (each
// loads the weights once and walks tiles), from the SM's registers and
// shared memory.  The first call raises the kernels' dynamic shared-memory
// limit (before any graph capture).
template <int T>
static int guided_resident_blocks() {
    auto* fn = k_material<T, false, true, kTcThreads>;
    DL_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGuidedSmem));
    DL_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    int dev = 0;
    DL_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    DL_CUDA(cudaGetDeviceProperties(&prop, dev));
    cudaFuncAttributes fa;
    DL_CUDA(cudaFuncGetAttributes(&fa, fn));
    const int regs_per_warp = ((fa.numRegs + 7) / 8) * 8 * 32;
    const int by_regs = prop.regsPerMultiprocessor / std::max(1, regs_per_warp * (kTcThreads / 32));
    const size_t smem = kGuidedSmem + fa.sharedSizeBytes + prop.reservedSharedMemPerBlock;
    const int by_smem = (int)(prop.sharedMemPerMultiprocessor / smem);
    return std::max(1, std::min(by_regs, by_smem));
}
static int guided_blocks(int sms) {
    static const int per_sm = std::min(std::min(guided_resident_blocks<MAT_DIFFUSE>(),
                                                guided_resident_blocks<MAT_MICROFACET>()),
                                       guided_resident_blocks<MAT_ANISO_GGX>());
    return sms * per_sm;
}

void render_guided(dl_scene* S, const dl_render_opts& o, dl_guide* G, float* d_film, bool train) {
    dl_context* ctx = S->ctx;
    cudaStream_t st = ctx->stream;
    const DevCamera& cam = S->dev.cam;
    RenderParams P;
    std::memset(&P, 0, sizeof(P));
    P.r0 = make_request(S, o);
    P.mode = 0;
    const unsigned long long npix = (unsigned long long)cam.w * cam.h;
    const int spp = std::max(o.spp, 1);
    const int chunk_spp = (int)std::max<size_t>(1, std::min<size_t>(spp, kSampleBufferBytes / (npix * 16)));
    const int64_t cap = pool_capacity(ctx, o.max_paths_in_flight, npix * (unsigned long long)chunk_spp);
    RenderBuffers& B = ctx->render;
    B.ensure(cap);
    B.grec.ensure((size_t)cap * 32);
    bind_pool(P, B);
    B.samples.ensure((size_t)npix * chunk_spp * 16);
    P.samples = B.samples.as<float4>();
    P.guided = 1;
    P.gnet.image = G->image.ptr;
    P.gnet.blocks = guided_blocks(ctx->num_sms);
    P.gnet.fraction = G->cfg.guide_fraction;
    P.gnet.max_depth = G->cfg.max_guided_depth;
    P.grec = B.grec.as<GuideRec>();
    const int64_t rec_cap = std::min<int64_t>((int64_t)G->cfg.batch * std::max(1, G->cfg.steps_per_pass), 1 << 23);
    GuideRecord* rec_half[2] = {nullptr, nullptr};
    if (train) {
        // a training step takes at most ceil(rec_cap / steps) records
        guide_reserve(G, (rec_cap + std::max(1, G->cfg.steps_per_pass) - 1) / std::max(1, G->cfg.steps_per_pass));
        // two halves: pass k writes half k % 2 while the training stream
        // learns from the other half (the previous pass)
        G->pass_recs.ensure(2 * (size_t)rec_cap * sizeof(GuideRecord));
        rec_half[0] = G->pass_recs.as<GuideRecord>();
        rec_half[1] = rec_half[0] + rec_cap;
        P.grecords = rec_half[0];  // non-null: the kernels write records
        P.grecord_cap = (int)rec_cap;
    }
    double kms[4] = {0, 0, 0, 0};
    int64_t launches = 0, iters = 0, records = 0;
    float train_ms = 0.f;
    RenderCounters acc;
    std::memset(&acc, 0, sizeof(acc));
    DL_CUDA(cudaEventRecord(ctx->ev0, st));
    FilmParams F = film_params(cam, P.r0, o.filter, d_film, P.samples, B.invalid.as<unsigned long long>());
    DL_CUDA(cudaMemsetAsync(F.invalid, 0, sizeof(unsigned long long), st));
    dim3 fgrid((F.cols + kFilmTile - 1) / kFilmTile, (F.rows + kFilmTile - 1) / kFilmTile);
    RenderCounters* hc = B.host_counters.as<RenderCounters>();
    int done = 0;
    bool trained[2] = {false, false};
    double guided_per_sample = 2.0 * (double)npix;  // guided vertices per sample per pixel: first guess
    cudaStream_t ts = G->train_stream;
    for (int pass = 0; done < spp; pass++) {
        int ns = std::min(std::min(pass == 0 ? 1 : (1 << (pass - 1)), spp - done), chunk_spp);
        // keep about rec_cap of the pass's guided vertices, spread over it
        const double expect = guided_per_sample * ns;
        const double frac = std::min(1.0, 0.9 * (double)rec_cap / std::max(expect, 1.0));
        const unsigned keep = (unsigned)std::max(1.0, frac * (double)(1u << 24));
        const int half = pass & 1;
        // the half this pass writes must be free of the training that read it
        if (train && trained[half]) DL_CUDA(cudaStreamWaitEvent(st, G->train_done[half], 0));
        run_wavefront(ctx, P, cap, false, false, kms, launches, iters, acc, npix * (unsigned long long)ns,
                      o.spp_offset + done, keep, rec_half[half]);
        const int64_t claimed = train ? (int64_t)hc->guide_next : 0;
        const int64_t nrec = std::min<int64_t>(claimed, rec_cap);
        if (train && claimed > 0)
            guided_per_sample = (double)claimed / ((double)keep / (double)(1u << 24)) / ns;
        F.nspp = ns;
        F.s_first = o.spp_offset + done;
        F.accumulate = done > 0;
        k_film_gather<<<fgrid, kFilmThreads, kFilmSmem, st>>>(F);
        launches += 1;
        DL_CUDA(cudaGetLastError());
        done += ns;
        const int steps = G->cfg.steps_per_pass;
        if (train && nrec >= 16 * (int64_t)std::max(1, steps) && done < spp) {
            // Adam steps on this pass's records, on the training stream: the
            // next pass renders meanwhile with the network as it changes (its
            // kernels sample and evaluate the same lobes, so every sample
            // stays unbiased).  Step k trains on records k, k + steps, ...:
            // every step sees the whole image.
            DL_CUDA(cudaEventRecord(G->pass_done[half], st));
            DL_CUDA(cudaStreamWaitEvent(ts, G->pass_done[half], 0));
            DL_CUDA(cudaEventRecord(G->t0, ts));
            for (int k = 0; k < steps; k++) {
                const int64_t cnt = (nrec - k + steps - 1) / steps;
                DL_CUDA(cudaMemsetAsync(G->grad.ptr, 0, kGuideParams * 4, ts));
                guide_gradient(G, rec_half[half] + k, cnt, steps, ts);
                guide_adam(G, ts);
            }
            DL_CUDA(cudaEventRecord(G->t1, ts));
            DL_CUDA(cudaEventRecord(G->train_done[half], ts));
            trained[half] = true;
        }
        records += nrec;
    }
    if (train && (trained[0] || trained[1])) {
        // the render ends when its last training round has ended
        DL_CUDA(cudaEventRecord(G->pass_done[0], ts));
        DL_CUDA(cudaStreamWaitEvent(st, G->pass_done[0], 0));
        DL_CUDA(cudaStreamSynchronize(ts));
        DL_CUDA(cudaEventElapsedTime(&train_ms, G->t0, G->t1));  // the last round's device time
    }
    unsigned long long* hinv =
        reinterpret_cast<unsigned long long*>(B.host_counters.as<char>() + sizeof(RenderCounters));
    DL_CUDA(cudaMemcpyAsync(hinv, F.invalid, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    DL_CUDA(cudaStreamSynchronize(st));
    acc.stat_invalid = *hinv;
    finish_stats(ctx, acc, *hinv, iters, launches, kms);
    ctx->stats.guide_records = records;
    ctx->stats.guide_train_ms = train_ms;
}

// Batch of requests in one wavefront: every pass renders, for each request
// with samples left, its next slice of samples per pixel; all requests' paths
// share the path pool and the material queues (each path carries its
// request), and after the pass one gather per request adds the slice to its
// film.  Slices are sized so a pass fits the sample buffer.
void render_batch(dl_context* ctx, const BatchItem* items, int n, bool count_traversal) {
    cudaStream_t st = ctx->stream;
    RenderBuffers& B = ctx->render;
    std::vector<int> done(n, 0);
    unsigned long long all = 0;
    for (int r = 0; r < n; r++)
        all += (unsigned long long)items[r].cam.w * items[r].cam.h * items[r].opts.spp;
    const unsigned long long budget = kSampleBufferBytes / 16;
    // slice of request r per pass: its share of the budget, at least one sample
    std::vector<int> slice(n);
    unsigned long long max_pass = 0;
    for (int r = 0; r < n; r++) {
        const unsigned long long npix = (unsigned long long)items[r].cam.w * items[r].cam.h;
        double share = all <= budget ? 1.0 : (double)budget / (double)all;
        slice[r] = std::max(1, std::min(items[r].opts.spp, (int)(items[r].opts.spp * share)));
        max_pass += npix * (unsigned long long)slice[r];
    }
    int64_t requested = 0;
    for (int r = 0; r < n; r++) requested = std::max<int64_t>(requested, items[r].opts.max_paths_in_flight);
    const int64_t cap = pool_capacity(ctx, requested, max_pass);
    B.ensure(cap);
    B.samples.ensure((size_t)std::max<unsigned long long>(max_pass, 1) * 16);
    B.requests.ensure(sizeof(DevRequest) * (size_t)std::max(n, 1));
    B.host_requests.ensure(sizeof(DevRequest) * (size_t)std::max(n, 1));
    DevRequest* hreq = B.host_requests.as<DevRequest>();
    RenderParams P;
    std::memset(&P, 0, sizeof(P));
    bind_pool(P, B);
    P.mode = 0;
    P.samples = B.samples.as<float4>();
    P.reqs = B.requests.as<DevRequest>();
    unsigned long long* d_invalid = B.invalid.as<unsigned long long>();
    double kms[4] = {0, 0, 0, 0};
    int64_t launches = 0, iters = 0;
    RenderCounters acc;
    std::memset(&acc, 0, sizeof(acc));
    DL_CUDA(cudaEventRecord(ctx->ev0, st));
    DL_CUDA(cudaMemsetAsync(d_invalid, 0, sizeof(unsigned long long), st));
    std::vector<int> active(n), ns(n);
    for (;;) {
        int na = 0;
        unsigned long long first = 0;
        for (int r = 0; r < n; r++) {
            if (done[r] >= items[r].opts.spp) continue;
            const unsigned long long npix = (unsigned long long)items[r].cam.w * items[r].cam.h;
            ns[na] = std::min(slice[r], items[r].opts.spp - done[r]);
            DevRequest R = make_request(items[r].scene, items[r].opts);
            R.sc.cam = items[r].cam;
            R.pid_first = first;
            R.spp_offset = items[r].opts.spp_offset + done[r];
            hreq[na] = R;
            active[na] = r;
            first += npix * (unsigned long long)ns[na];
            na++;
        }
        if (na == 0) break;
        // the pass's request table; the copy is ordered before the pass's kernels
        DL_CUDA(cudaMemcpyAsync(B.requests.ptr, hreq, sizeof(DevRequest) * na, cudaMemcpyHostToDevice, st));
        P.num_reqs = na;
        run_wavefront(ctx, P, cap, true, count_traversal, kms, launches, iters, acc, first, 0, 1u << 24);
        for (int a = 0; a < na; a++) {
            const int r = active[a];
            const DevCamera& cam = items[r].cam;
            FilmParams F = film_params(cam, hreq[a], items[r].opts.filter, items[r].d_film,
                                       P.samples + hreq[a].pid_first, d_invalid);
            F.nspp = ns[a];
            F.s_first = hreq[a].spp_offset;
            F.accumulate = done[r] > 0;
            dim3 fgrid((F.cols + kFilmTile - 1) / kFilmTile, (F.rows + kFilmTile - 1) / kFilmTile);
            k_film_gather<<<fgrid, kFilmThreads, kFilmSmem, st>>>(F);
            launches += 1;
            DL_CUDA(cudaGetLastError());
            done[r] += ns[a];
        }
        // host_requests is rewritten next pass: wait for this pass's copy
        DL_CUDA(cudaStreamSynchronize(st));
    }
    unsigned long long* hinv =
        reinterpret_cast<unsigned long long*>(B.host_counters.as<char>() + sizeof(RenderCounters));
    DL_CUDA(cudaMemcpyAsync(hinv, d_invalid, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    DL_CUDA(cudaStreamSynchronize(st));
    acc.stat_invalid = *hinv;
    finish_stats(ctx, acc, *hinv, iters, launches, kms);
}

// Li of explicit paths with every piece of path state in caller-provided
// device memory (`pool`, laid out below) and no allocation of any kind: no
// cudaMalloc, no pinned staging (the counters are read back into a stack
// copy), no graph.  Used by the allocation-free entry point.
constexpr size_t kCounterBytes = (sizeof(RenderCounters) + 255) / 256 * 256;
size_t fixed_pool_bytes(int64_t slots) { return kSlotBytes * (size_t)slots + kCounterBytes; }

// Failures throw dl::Error with the status and message that run_wavefront
// gives for the same condition.
void render_li_fixed(dl_scene* S, const dl_render_opts& o, void* pool, int64_t slots, int64_t li_n,
                     const int* d_xys, float* d_L, float* d_pos) {
    dl_context* ctx = S->ctx;
    cudaStream_t st = ctx->stream;
    RenderParams P;
    std::memset(&P, 0, sizeof(P));
    P.r0 = make_request(S, o);
    P.mode = 1;
    P.capacity = (int)slots;
    size_t c = (size_t)slots;
    char* b = static_cast<char*>(pool);
    P.cnt = reinterpret_cast<RenderCounters*>(b);
    b += kCounterBytes;
    P.rec = reinterpret_cast<SlotRec*>(b); b += 128 * c;
    float4** f4[] = {&P.sh_o, &P.sh_d, &P.sh_c};
    for (float4** f : f4) {
        *f = reinterpret_cast<float4*>(b);
        b += 16 * c;
    }
    P.pos = reinterpret_cast<float2*>(b); b += 8 * c;
    int** iq[] = {&P.ext_q[0], &P.ext_q[1], &P.mat_q[0], &P.mat_q[1], &P.mat_q[2], &P.mat_q[3], &P.mat_q[4],
                  &P.mat_q[5]};
    for (int** q : iq) {
        *q = reinterpret_cast<int*>(b);
        b += 4 * c;
    }
    P.xys = d_xys;
    P.li_L = d_L;
    P.li_pos = d_pos;
    int64_t cap = std::min<int64_t>(slots, ((li_n + 31) / 32) * 32);
    const int sms = ctx->num_sms > 0 ? ctx->num_sms : 152;
    DL_CUDA(cudaMemsetAsync(P.cnt, 0, sizeof(RenderCounters), st));
    // pass values from the stack (a pageable copy: staged before it returns)
    PassValues pv;
    pv.total = (unsigned long long)li_n;
    pv.spp_offset = 0;
    pv.keep = 1u << 24;
    pv.recs = nullptr;
    DL_CUDA(cudaMemcpyAsync(&P.cnt->pass_total, &pv, sizeof(pv), cudaMemcpyHostToDevice, st));
    k_init<false><<<sms * 16, 128, 0, st>>>(P, (int)cap);
    RenderCounters hc;
    int64_t iters = 0;
    const TuneParams tp;  // default launch shape
    for (;;) {
        for (int k = 0; k < tp.iters_per_graph; k++)
            launch_iteration<false>(P, k & 1, st, sms, tp, false, nullptr, nullptr);
        iters += tp.iters_per_graph;
        DL_CUDA(cudaGetLastError());
        DL_CUDA(cudaMemcpyAsync(&hc, P.cnt, sizeof(RenderCounters), cudaMemcpyDeviceToHost, st));
        DL_CUDA(cudaStreamSynchronize(st));
        if (hc.err & kErrBounds) throw Error(DL_ERR_QUEUE_OVERFLOW, kBoundsMessage);
        if (hc.err & kErrTensorWait) throw Error(DL_ERR_TIMEOUT, "tensor-core wait timed out in a guided kernel");
        if (hc.err) throw Error(DL_ERR_QUEUE_OVERFLOW, "traversal stack overflow");
        if (hc.ext[0] == 0 && hc.shadow[0] == 0 && hc.next_path >= (unsigned long long)li_n) break;
        if (iters > 1000000) throw Error(DL_ERR_TIMEOUT, "render did not converge");
    }
}

void resolve_film(dl_scene* S, const float* d_film, int filter, float* d_rgb) {
    resolve_film_cam(S->dev.cam, S->ctx->stream, d_film, filter, d_rgb);
}

void resolve_film_cam(const DevCamera& cam, cudaStream_t st, const float* d_film, int filter, float* d_rgb) {
    int b = filter == DL_FILTER_BOX ? 0 : 2;
    int n = cam.w * cam.h;
    k_resolve<<<(n + 255) / 256, 256, 0, st>>>(reinterpret_cast<const float4*>(d_film),
                                                         cam.w + 2 * b, b, cam.w, cam.h, d_rgb);
    DL_CUDA(cudaGetLastError());
}

}  // namespace dl

namespace dl {

// ------------------------------------------------- rays through k_traverse
// Ray batches through the renderer's own traversal kernels, the exact
// template instances a single-scene render launches (k_traverse<false,
// false, false> for closest hits, k_traverse<false, true, false> for shadow
// rays) with the context's launch shape, so that ray-level parity tests
// exercise the kernels dl_render runs.  Each ray gets a path slot: its ray
// record (closest hit) or its shadow-queue entry with a unit contribution
// aimed at sample i (any hit), in queue order 0..n-1.

__global__ void k_wavefront_rays_setup(RenderParams P, const float4* __restrict__ rays, int n, int any) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 o = rays[2 * i], d = rays[2 * i + 1];
        if (any) {
            P.sh_o[i] = make_float4(o.x, o.y, o.z, __int_as_float(0));
            P.sh_d[i] = d;
            P.sh_c[i] = make_float4(1.f, 1.f, 1.f, __int_as_float(-1 - i));
            P.li_L[3 * i] = 0.f;
            P.li_L[3 * i + 1] = 0.f;
            P.li_L[3 * i + 2] = 0.f;
        } else {
            RayRec r;
            r.o = make_float4(o.x, o.y, o.z, __int_as_float(0));
            r.d = d;
            P.rec[i].ray = r;
            P.ext_q[0][i] = i;
        }
    }
}

// hits (n x float4: t, u, v, original triangle id bits, -1 = miss) from the
// hit records; occluded flags from the delivered unit contributions.
__global__ void k_wavefront_rays_out(RenderParams P, int n, int any, float4* __restrict__ hits,
                                     uint8_t* __restrict__ occ) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (any) {
            occ[i] = P.li_L[3 * i] == 0.f ? 1 : 0;
        } else {
            const float4 h = P.rec[i].hit.h;
            const int tri = __float_as_int(h.w);
            const int prim = tri >= 0 ? __float_as_int(__ldg(P.r0.sc.tris + 3 * tri).w) : -1;
            hits[i] = make_float4(tri >= 0 ? h.x : 0.f, tri >= 0 ? h.y : 0.f, tri >= 0 ? h.z : 0.f,
                                  __int_as_float(prim));
        }
    }
}

size_t wavefront_rays_bytes(int64_t n) {
    return kCounterBytes + 128 * (size_t)n + 3 * 16 * (size_t)n + 12 * (size_t)n +
           4 * (size_t)n * (2 + kNumMaterialTypes + 1);
}

// d_rays: n x 8 floats (o, tmin, d, tmax) with tmin = kRayEps for every ray
// (the renderer's constant ray start); `work` holds wavefront_rays_bytes(n).
void trace_wavefront_launch(dl_scene* S, bool any, const float* d_rays, int64_t n, float* d_hits, uint8_t* d_occ,
                            void* work) {
    dl_context* ctx = S->ctx;
    cudaStream_t st = ctx->stream;
    if (n == 0) return;
    RenderParams P;
    std::memset(&P, 0, sizeof(P));
    dl_render_opts o;
    std::memset(&o, 0, sizeof(o));
    P.r0 = make_request(S, o);
    P.mode = 1;
    P.capacity = (int)n;
    char* b = static_cast<char*>(work);
    P.cnt = reinterpret_cast<RenderCounters*>(b);
    b += kCounterBytes;
    P.rec = reinterpret_cast<SlotRec*>(b);
    b += 128 * (size_t)n;
    float4** f4[] = {&P.sh_o, &P.sh_d, &P.sh_c};
    for (float4** f : f4) {
        *f = reinterpret_cast<float4*>(b);
        b += 16 * (size_t)n;
    }
    P.li_L = reinterpret_cast<float*>(b);
    b += 12 * (size_t)n;
    int** iq[] = {&P.ext_q[0], &P.ext_q[1], &P.mat_q[0], &P.mat_q[1], &P.mat_q[2], &P.mat_q[3], &P.mat_q[4],
                  &P.mat_q[5]};
    for (int** q : iq) {
        *q = reinterpret_cast<int*>(b);
        b += 4 * (size_t)n;
    }
    DL_CUDA(cudaMemsetAsync(P.cnt, 0, sizeof(RenderCounters), st));
    const int ni = (int)n;
    const unsigned long long total = (unsigned long long)n;  // path indices of the shadow targets: 0..n-1
    DL_CUDA(cudaMemcpyAsync(any ? &P.cnt->shadow[0] : &P.cnt->ext[0], &ni, sizeof(int), cudaMemcpyHostToDevice, st));
    DL_CUDA(cudaMemcpyAsync(&P.cnt->pass_total, &total, sizeof(total), cudaMemcpyHostToDevice, st));
    const int sms = ctx->num_sms > 0 ? ctx->num_sms : 152;
    const int g = (int)std::min<int64_t>((n + 127) / 128, (int64_t)sms * 16);
    k_wavefront_rays_setup<<<g, 128, 0, st>>>(P, reinterpret_cast<const float4*>(d_rays), ni, any ? 1 : 0);
    const int tb = sms * ctx->tune.trav_ctas_per_sm;
    if (any) k_traverse<false, true, false><<<tb, 128, 0, st>>>(P, 0);
    else k_traverse<false, false, false><<<tb, 128, 0, st>>>(P, 0);
    k_wavefront_rays_out<<<g, 128, 0, st>>>(P, ni, any ? 1 : 0, reinterpret_cast<float4*>(d_hits), d_occ);
    DL_CUDA(cudaGetLastError());
    unsigned int err = 0;
    DL_CUDA(cudaMemcpyAsync(&err, &P.cnt->err, sizeof(err), cudaMemcpyDeviceToHost, st));
    DL_CUDA(cudaStreamSynchronize(st));
    if (err & kErrBounds) throw Error(DL_ERR_QUEUE_OVERFLOW, kBoundsMessage);
    if (err) throw Error(DL_ERR_QUEUE_OVERFLOW, "traversal stack overflow");
}

}  // namespace dl

namespace dl {

// ------------------------------------------------------- emitter queries
// Scene::sampleEmitterDirection without the visibility test, at given
// points, normals and 2D samples, by the device function the material
// kernels run (an envmap pick draws its three numbers from a pcg32 seeded
// with the query index); `light` receives the picked emitter.
__global__ void __launch_bounds__(128) k_emitter_query(DevRequest R, int n, const float* __restrict__ pts,
                                                        const float* __restrict__ nrm, const float* __restrict__ smp,
                                                        float* __restrict__ out, int* __restrict__ light) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float3 p = f3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
        const float3 nn = f3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
        const float2 s = make_float2(smp[2 * i], smp[2 * i + 1]);
        float sx = s.x;
        light[i] = R.sc.num_lights > 0 ? pick_light(R, sx) : -1;
        Pcg32 g;
        g.seed((unsigned long long)i, 7ull);
        float3 d;
        float dist, pdf;
        bool delta;
        const float3 spec = sample_emitter(R, p, nn, s, g, d, dist, pdf, delta);
        float* o = out + 8 * (size_t)i;
        o[0] = d.x;
        o[1] = d.y;
        o[2] = d.z;
        o[3] = dist;
        o[4] = pdf;
        o[5] = spec.x;
        o[6] = spec.y;
        o[7] = spec.z;
    }
}

void emitter_query(dl_scene* S, uint32_t flags, int64_t n, const float* pts, const float* nrm, const float* smp,
                   float* d, float* dist, float* pdf, float* spec, int32_t* light) {
    if (n == 0) return;
    dl_context* ctx = S->ctx;
    cudaStream_t st = ctx->stream;
    dl_render_opts o;
    std::memset(&o, 0, sizeof(o));
    o.flags = flags;
    const DevRequest R = make_request(S, o);
    const size_t f = sizeof(float) * (size_t)n;
    DevBuf buf;
    buf.ensure(f * (3 + 3 + 2 + 8 + 1));
    float* d_pts = buf.as<float>();
    float* d_nrm = d_pts + 3 * n;
    float* d_smp = d_nrm + 3 * n;
    float* d_out = d_smp + 2 * n;
    int* d_light = reinterpret_cast<int*>(d_out + 8 * n);
    DL_CUDA(cudaMemcpyAsync(d_pts, pts, 3 * f, cudaMemcpyHostToDevice, st));
    DL_CUDA(cudaMemcpyAsync(d_nrm, nrm, 3 * f, cudaMemcpyHostToDevice, st));
    DL_CUDA(cudaMemcpyAsync(d_smp, smp, 2 * f, cudaMemcpyHostToDevice, st));
    const int sms = ctx->num_sms > 0 ? ctx->num_sms : 152;
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 127) / 128, (int64_t)sms * 8));
    k_emitter_query<<<g, 128, 0, st>>>(R, (int)n, d_pts, d_nrm, d_smp, d_out, d_light);
    DL_CUDA(cudaGetLastError());
    std::vector<float> h((size_t)n * 8);
    DL_CUDA(cudaMemcpyAsync(h.data(), d_out, 8 * f, cudaMemcpyDeviceToHost, st));
    DL_CUDA(cudaMemcpyAsync(light, d_light, f, cudaMemcpyDeviceToHost, st));
    DL_CUDA(cudaStreamSynchronize(st));
    for (int64_t i = 0; i < n; i++) {
        const float* q = &h[8 * (size_t)i];
        for (int k = 0; k < 3; k++) {
            d[3 * i + k] = q[k];
            spec[3 * i + k] = q[5 + k];
        }
        dist[i] = q[3];
        pdf[i] = q[4];
    }
}

}  // namespace dl
