// Test harness over the reference's own CPU path (xuxmin/DrawLab), compiled
// from the reference sources where they lie by oracle/build.py into
// oracle/_ref/libdlref.so.  TEST INFRASTRUCTURE ONLY: tests and the golden
// fixture generator call it to pin the CPU restatement (oracle/oracle.cpp);
// nothing in the product links it.
//
// It builds a drawlab::Scene from the dl_*_desc arrays of include/drawlab.h
// through the reference's ObjectFactory, then exposes:
//   ref_trace_closest / ref_trace_any  -> OCTree::recursiveIntersect /
//       recursiveAnyhit (src/tracer/accel/octree.cpp:53-133)
//   ref_render_blocks -> the CPURenderer block loop
//       (src/tracer/backend/cpu_renderer.cpp:22-117) on std::thread workers
//       in place of tbb::parallel_for
//   ref_li            -> PathIntegrator::Li (src/tracer/integrator/path.cpp:13)
//       for given (x, y, s) paths, each with its own pcg32 stream
//   ref_bsdf_query / ref_emitter_sample -> BSDF::eval/pdf/sample and
//       Scene::sampleEmitterDirection on given inputs.
// Private members are reached by compiling the reference headers with
// `private`/`protected` redefined to `public` (layout is unchanged).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#define private public
#define protected public
#include "core/bitmap/block.h"
#include "core/parser/object.h"
#include "core/parser/proplist.h"
#include "tracer/bsdf.h"
#include "tracer/camera.h"
#include "tracer/emitter.h"
#include "tracer/integrator.h"
#include "tracer/mesh.h"
#include "tracer/octree.h"
#include "tracer/rfilter.h"
#include "tracer/sampler.h"
#include "tracer/scene.h"
#undef private
#undef protected

#include <pcg32.h>

#include "../include/drawlab.h"

using namespace drawlab;

namespace {

struct ArrayMesh : public Mesh {
    explicit ArrayMesh(const dl_mesh_desc& d) {
        m_V.assign(d.positions, d.positions + 3 * d.num_vertices);
        if (d.normals) m_N.assign(d.normals, d.normals + 3 * d.num_vertices);
        if (d.texcoords) m_UV.assign(d.texcoords, d.texcoords + 2 * d.num_vertices);
        m_F.assign(d.indices, d.indices + 3 * d.num_triangles);
        for (int64_t i = 0; i < d.num_vertices; i++)
            m_bbox.expandBy(Point3f(m_V[3 * i], m_V[3 * i + 1], m_V[3 * i + 2]));
    }
};

struct RefScene {
    Scene* scene = nullptr;
    OCTree* tree = nullptr;
    std::vector<const Mesh*> mesh_of_desc;   // desc index -> mesh
    std::map<const Mesh*, int64_t> prim_offset;
    std::vector<int64_t> accel_prim_offset;  // accel mesh index -> global prim offset
    int width = 0, height = 0;
};

Vector3f v3(const float* p) { return Vector3f(p[0], p[1], p[2]); }
Color3f c3(const float* p) { return Color3f(p[0], p[1], p[2]); }

BSDF* make_bsdf(const dl_material_desc& m) {
    PropertyList pl;
    const char* name = nullptr;
    switch (m.type) {
        case DL_MAT_DIFFUSE: name = "diffuse"; pl.setColor("albedo", c3(m.albedo)); break;
        case DL_MAT_MIRROR: name = "mirror"; break;
        case DL_MAT_DIELECTRIC:
            name = "dielectric";
            pl.setFloat("intIOR", m.int_ior);
            pl.setFloat("extIOR", m.ext_ior);
            break;
        case DL_MAT_MICROFACET:
            name = "microfacet";
            pl.setFloat("alpha", m.alpha[0]);
            pl.setFloat("intIOR", m.int_ior);
            pl.setFloat("extIOR", m.ext_ior);
            pl.setColor("kd", c3(m.albedo));
            break;
        case DL_MAT_ANISO_GGX:
            // The reference CPU backend's aniso_ggx is a stub returning 0
            // (src/tracer/bsdf/aniso_ggx.cpp:29-41); it is built as-is.
            name = "aniso_ggx";
            pl.setColor("pd", c3(m.albedo));
            pl.setColor("ps", c3(m.specular));
            pl.setColor("axay", Color3f(m.alpha[0], m.alpha[1], 0.f));
            break;
        default: return nullptr;
    }
    Object* o = ObjectFactory::createInstance(name, pl);
    o->activate();
    return static_cast<BSDF*>(o);
}

thread_local std::string g_err;

struct IndependentLayout : public Sampler {
    pcg32 m_random;
};

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

void* ref_scene_create(const dl_mesh_desc* meshes, int32_t nm, const dl_material_desc* mats,
                       int32_t nmat, const dl_light_desc* lights, int32_t nl,
                       const dl_camera_desc* cam, int32_t filter, int32_t spp, int32_t normals) {
    try {
        auto* rs = new RefScene();
        rs->scene = new Scene(PropertyList());
        std::vector<Mesh*> built(nm, nullptr);
        for (int i = 0; i < nm; i++) {
            auto* m = new ArrayMesh(meshes[i]);
            if (meshes[i].material < 0 || meshes[i].material >= nmat) throw Exception("bad material");
            m->addChild(make_bsdf(mats[meshes[i].material]));
            built[i] = m;
        }
        // Meshes are added in array order (that is the octree's triangle
        // order), each with its area emitter; point lights follow.  The
        // scene's emitter order (Scene::addChild, src/tracer/scene/scene.cpp:
        // 36-81) must then equal the light-array order, else the scene is
        // rejected: area lights in mesh order first, point lights last.
        std::vector<int> order;
        for (int l = 0; l < nl; l++) {
            const dl_light_desc& L = lights[l];
            if (L.type == DL_LIGHT_AREA) {
                PropertyList pl;
                pl.setColor("radiance", c3(L.radiance));
                Object* e = ObjectFactory::createInstance("area", pl);
                e->activate();
                if (L.mesh < 0 || L.mesh >= nm) throw Exception("bad light mesh");
                built[L.mesh]->addChild(e);
            } else if (L.type != DL_LIGHT_POINT) {
                throw Exception("light type not available in the reference CPU backend");
            }
        }
        for (int i = 0; i < nm; i++) {
            built[i]->activate();
            rs->scene->addChild(built[i]);
            if (meshes[i].light >= 0) order.push_back(meshes[i].light);
        }
        for (int l = 0; l < nl; l++) {
            const dl_light_desc& L = lights[l];
            if (L.type != DL_LIGHT_POINT) continue;
            PropertyList pl;
            pl.setColor("intensity", c3(L.radiance));
            pl.setPoint("position", Point3f(L.position[0], L.position[1], L.position[2]));
            Object* e = ObjectFactory::createInstance("point", pl);
            e->activate();
            rs->scene->addChild(e);
            order.push_back(l);
        }
        for (int l = 0; l < (int)order.size(); l++)
            if (order[l] != l) throw Exception("light order not representable by the reference");

        PropertyList cp;
        cp.setInteger("width", cam->width);
        cp.setInteger("height", cam->height);
        cp.setFloat("fov", cam->fov);
        Object* camera = nullptr;
        if (cam->type == DL_CAMERA_VIRTUAL) {
            cp.setVector("eye", v3(cam->eye));
            cp.setVector("lookat", v3(cam->lookat));
            cp.setVector("up", v3(cam->up));
            camera = ObjectFactory::createInstance("virtual", cp);
        } else if (cam->type == DL_CAMERA_PERSPECTIVE) {
            cp.setFloat("nearClip", cam->near_clip);
            cp.setFloat("farClip", cam->far_clip);
            Matrix4f m;
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++) m[i][j] = cam->transform[4 * i + j];
            cp.setTransform("toWorld", Transform(m));
            camera = ObjectFactory::createInstance("perspective", cp);
        } else {
            throw Exception("camera type not available in the reference CPU backend");
        }
        Object* rf = ObjectFactory::createInstance(filter == DL_FILTER_BOX ? "box" : "gaussian",
                                                   PropertyList());
        rf->activate();
        camera->addChild(rf);
        camera->activate();
        rs->scene->addChild(camera);
        PropertyList sp;
        sp.setInteger("sampleCount", spp);
        Object* sampler = ObjectFactory::createInstance("independent", sp);
        sampler->activate();
        rs->scene->addChild(sampler);
        Object* integ = ObjectFactory::createInstance(normals ? "normals" : "path", PropertyList());
        integ->activate();
        rs->scene->addChild(integ);
        rs->scene->activate();

        rs->tree = static_cast<OCTree*>(rs->scene->m_accel);
        int64_t off = 0;
        for (int i = 0; i < nm; i++) {
            rs->prim_offset[built[i]] = off;
            rs->mesh_of_desc.push_back(built[i]);
            off += meshes[i].num_triangles;
        }
        for (Mesh* m : rs->tree->m_meshPtrs) rs->accel_prim_offset.push_back(rs->prim_offset[m]);
        rs->width = cam->width;
        rs->height = cam->height;
        return rs;
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

void ref_scene_destroy(void* p) {
    // The reference scene owns raw pointers in a way that double-frees shared
    // objects (Mesh deletes its BSDF and emitter); the harness leaks it.
    (void)p;
}

static void load_ray(const float* r, Ray3f& ray) {
    ray = Ray3f(Point3f(r[0], r[1], r[2]), Vector3f(r[4], r[5], r[6]), r[3], r[7]);
}

int ref_trace_closest(void* p, const float* rays, int64_t n, int32_t* prim, float* t,
                      float* u, float* v, int32_t threads) {
    auto* rs = static_cast<RefScene*>(p);
    auto work = [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) {
            Ray3f ray;
            load_ray(rays + 8 * i, ray);
            Point2f uv(0, 0);
            float tt = 0;
            std::pair<int, int> f(-1, -1);
            bool hit = rs->tree->recursiveIntersect(rs->tree->m_root, ray, uv, tt, f);
            if (hit) {
                prim[i] = (int32_t)(rs->accel_prim_offset[f.first] + f.second);
                t[i] = tt;
                u[i] = uv.x();
                v[i] = uv.y();
            } else {
                prim[i] = -1;
                t[i] = u[i] = v[i] = 0.f;
            }
        }
    };
    int T = std::max(1, threads);
    std::vector<std::thread> th;
    for (int k = 0; k < T; k++) th.emplace_back(work, n * k / T, n * (k + 1) / T);
    for (auto& x : th) x.join();
    return 0;
}

int ref_trace_any(void* p, const float* rays, int64_t n, uint8_t* occ, int32_t threads) {
    auto* rs = static_cast<RefScene*>(p);
    auto work = [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) {
            Ray3f ray;
            load_ray(rays + 8 * i, ray);
            occ[i] = rs->scene->rayIntersect(ray) ? 1 : 0;
        }
    };
    int T = std::max(1, threads);
    std::vector<std::thread> th;
    for (int k = 0; k < T; k++) th.emplace_back(work, n * k / T, n * (k + 1) / T);
    for (auto& x : th) x.join();
    return 0;
}

// CPURenderer::renderBlock (src/tracer/backend/cpu_renderer.cpp:22-55).
static void render_block(const Scene* scene, Sampler* sampler, ImageBlock& block) {
    const Camera* camera = scene->getCamera();
    const Integrator* integrator = scene->getIntegrator();
    Point2i offset = block.getOffset();
    Vector2i size = block.getSize();
    block.clear();
    for (int y = 0; y < size.y(); ++y)
        for (int x = 0; x < size.x(); ++x)
            for (uint32_t i = 0; i < sampler->getSampleCount(); ++i) {
                Point2f pixelSample =
                    Point2f((float)(x + offset.x()), (float)(y + offset.y())) + sampler->next2D();
                Point2f apertureSample = sampler->next2D();
                Ray3f ray;
                Color3f value = camera->sampleRay(ray, pixelSample, apertureSample);
                value *= integrator->Li(scene, sampler, ray);
                block.put(pixelSample, value);
            }
}

static void film_to_outputs(const ImageBlock& film, float* rgb_out, float* film_out) {
    int b = film.getBorderSize();
    Vector2i sz = film.getSize();
    if (rgb_out)
        for (int y = 0; y < sz.y(); y++)
            for (int x = 0; x < sz.x(); x++) {
                Color3f c = film.coeffRef(y + b, x + b).divideByFilterWeight();
                float* o = rgb_out + 3 * ((int64_t)y * sz.x() + x);
                o[0] = c[0]; o[1] = c[1]; o[2] = c[2];
            }
    if (film_out) {
        int rows = sz.y() + 2 * b, cols = sz.x() + 2 * b;
        for (int y = 0; y < rows; y++)
            for (int x = 0; x < cols; x++) {
                const Color4f& c = film.coeffRef(y, x);
                float* o = film_out + 4 * ((int64_t)y * cols + x);
                o[0] = c[0]; o[1] = c[1]; o[2] = c[2]; o[3] = c[3];
            }
    }
}

// The reference CPU render: spiral 32x32 blocks, one pcg32 stream per block
// seeded with the block offset, per-thread sampler clone, Gaussian/box splat
// and a locked merge (cpu_renderer.cpp:57-135, block.cpp:81-177).
// `max_blocks` > 0 renders only the first max_blocks blocks of the spiral.
int ref_render_blocks(void* p, int32_t threads, int32_t max_blocks, float* rgb_out,
                      float* film_out, double* seconds) {
    auto* rs = static_cast<RefScene*>(p);
    Scene* scene = rs->scene;
    const Camera* camera = scene->getCamera();
    Vector2i outputSize = camera->getOutputSize();
    ImageBlock film(outputSize, camera->getReconstructionFilter());
    film.clear();
    const int BLOCK_SIZE = 32;
    BlockGenerator gen(outputSize, BLOCK_SIZE);
    int total = gen.getBlockCount();
    if (max_blocks > 0 && max_blocks < total) total = max_blocks;
    std::atomic<int> taken(0);
    auto t0 = std::chrono::steady_clock::now();
    auto worker = [&]() {
        ImageBlock block(Vector2i(BLOCK_SIZE), camera->getReconstructionFilter());
        std::unique_ptr<Sampler> sampler(scene->getSampler()->clone());
        while (true) {
            if (taken.fetch_add(1) >= total) break;
            if (!gen.next(block)) break;
            sampler->prepare(block);
            render_block(scene, sampler.get(), block);
            film.put(block);
        }
    };
    int T = std::max(1, threads);
    std::vector<std::thread> th;
    for (int k = 0; k < T; k++) th.emplace_back(worker);
    for (auto& x : th) x.join();
    auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    film_to_outputs(film, rgb_out, film_out);
    return 0;
}

static inline uint64_t splitmix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// Li of explicit paths; each path (x, y, s) seeds its own pcg32 stream with
// initseq = s*W*H + y*W + x and initstate = splitmix64(initseq ^ splitmix64(seed)),
// the same per-path streams as the GPU renderer and the oracle.
int ref_li(void* p, uint64_t seed, int64_t n, const int32_t* xys, float* L, float* pos,
           int32_t threads) {
    auto* rs = static_cast<RefScene*>(p);
    const Scene* scene = rs->scene;
    const uint64_t W = (uint64_t)rs->width, H = (uint64_t)rs->height;
    const uint64_t sseed = splitmix64(seed);
    auto work = [&](int64_t b, int64_t e) {
        std::unique_ptr<Sampler> sampler(scene->getSampler()->clone());
        auto* ind = sampler.get();
        for (int64_t i = b; i < e; i++) {
            int x = xys[3 * i], y = xys[3 * i + 1], s = xys[3 * i + 2];
            uint64_t seq = (uint64_t)s * W * H + (uint64_t)y * W + (uint64_t)x;
            // Independent is declared only inside its .cpp: its pcg32 member
            // (src/tracer/sampler/independent.cpp:56) directly follows the
            // Sampler base, which IndependentLayout mirrors.
            static_cast<IndependentLayout*>(ind)->m_random.seed(splitmix64(seq ^ sseed), seq);
            Point2f pixelSample = Point2f((float)x, (float)y) + ind->next2D();
            Point2f apertureSample = ind->next2D();
            Ray3f ray;
            Color3f value = scene->getCamera()->sampleRay(ray, pixelSample, apertureSample);
            value *= scene->getIntegrator()->Li(scene, ind, ray);
            L[3 * i] = value[0]; L[3 * i + 1] = value[1]; L[3 * i + 2] = value[2];
            if (pos) { pos[2 * i] = pixelSample.x(); pos[2 * i + 1] = pixelSample.y(); }
        }
    };
    int T = std::max(1, threads);
    std::vector<std::thread> th;
    for (int k = 0; k < T; k++) th.emplace_back(work, n * k / T, n * (k + 1) / T);
    for (auto& x : th) x.join();
    return 0;
}

// BSDF::eval / pdf / sample on given local directions (bsdf.h:46-110).
// Per query i: wi, wo (3 floats each), sample (2 floats).  Outputs: eval (3),
// pdf (1), sampled wo (3), sample weight (3), sample eta (1), measure (1 int).
int ref_bsdf_query(const dl_material_desc* m, int64_t n, const float* wi, const float* wo,
                   const float* smp, float* eval, float* pdf, float* s_wo, float* s_w,
                   float* s_eta, int32_t* s_measure) {
    BSDF* bsdf = make_bsdf(*m);
    if (!bsdf) return 1;
    Intersection its;
    for (int64_t i = 0; i < n; i++) {
        BSDFQueryRecord q(its, v3(wi + 3 * i), v3(wo + 3 * i), ESolidAngle);
        Color3f e = bsdf->eval(q);
        eval[3 * i] = e[0]; eval[3 * i + 1] = e[1]; eval[3 * i + 2] = e[2];
        pdf[i] = bsdf->pdf(q);
        BSDFQueryRecord s(its, v3(wi + 3 * i));
        Color3f w = bsdf->sample(s, Point2f(smp[2 * i], smp[2 * i + 1]));
        s_wo[3 * i] = s.wo[0]; s_wo[3 * i + 1] = s.wo[1]; s_wo[3 * i + 2] = s.wo[2];
        s_w[3 * i] = w[0]; s_w[3 * i + 1] = w[1]; s_w[3 * i + 2] = w[2];
        s_eta[i] = s.eta;
        s_measure[i] = (int32_t)s.measure;
    }
    return 0;
}

// Frame(n) (include/core/math/frame.h:104-123): n (3) -> t (3), b (3).
int ref_frame(int64_t n, const float* nrm, float* t, float* b) {
    for (int64_t i = 0; i < n; i++) {
        Frame f(Normal3f(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]));
        for (int k = 0; k < 3; k++) { t[3 * i + k] = f.t[k]; b[3 * i + k] = f.b[k]; }
    }
    return 0;
}

// Scene::sampleEmitterDirection (scene.cpp:139-170) at points p with shading
// normal n (shading frame Frame(n)): outputs d (3), dist, pdf, spectrum (3,
// visibility applied).
int ref_emitter_sample(void* p, int64_t n, const float* pts, const float* nrm, const float* smp,
                       float* d, float* dist, float* pdf, float* spec) {
    auto* rs = static_cast<RefScene*>(p);
    for (int64_t i = 0; i < n; i++) {
        Intersection its;
        its.p = Point3f(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
        its.shFrame = Frame(Normal3f(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]));
        its.geoFrame = its.shFrame;
        DirectionSample ds;
        Color3f sp;
        rs->scene->sampleEmitterDirection(its, Point2f(smp[2 * i], smp[2 * i + 1]), ds, sp);
        for (int k = 0; k < 3; k++) { d[3 * i + k] = ds.d[k]; spec[3 * i + k] = sp[k]; }
        dist[i] = ds.dist;
        pdf[i] = ds.pdf;
    }
    return 0;
}

// The pcg32 the reference build links (oracle/ref_shim/pcg32.h, standing in
// for the un-vendored ext/pcg32 submodule): n outputs of seed(initstate,
// initseq) as nextUInt and as nextFloat.
int ref_pcg32(uint64_t initstate, uint64_t initseq, int32_t n, uint32_t* out, float* out_float) {
    pcg32 a(initstate, initseq), b(initstate, initseq);
    for (int32_t i = 0; i < n; i++) {
        out[i] = a.nextUInt();
        out_float[i] = b.nextFloat();
    }
    return 0;
}

}  // extern "C"
