// Reference harness, host set-up of the OptiX-only emitters and cameras
// (TEST INFRASTRUCTURE ONLY; never shipped).
//
// refx_env_tables drives the reference's own EnvironmentMap::activate /
// build_alias_map (src/tracer/emitter/envmap.cpp:59-141), compiled from
// where it lies, on a bitmap held in memory.  refx_opencv_setup drives the
// reference's OpencvCamera constructor and getOptixCamera
// (src/tracer/camera/opencv.cpp:10-83): the inverse extrinsic and eye the
// OptiX camera receives.  The reference's emitter takes its bitmap from a
// "bitmap" texture that loads a file through stb_image / OpenEXR (absent
// here); this harness registers its own "bitmap" texture class that hands
// out an in-memory Bitmap instead, so the factory path of the constructor
// runs unchanged.  The emitter keeps its tables private; the harness reads
// them by compiling the file with private members made public.
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "core/bitmap/bitmap.h"
#include "core/parser/object.h"
#include "core/parser/proplist.h"
#include "core/utils/timer.h"
#include "optix/host/cuda_buffer.h"
#include "optix/light/envmap.h"
#include "tracer/camera.h"
#include "tracer/emitter.h"
// tracer/texture.h has no include guard: envmap.cpp includes it below

#define private public
#include "src/tracer/emitter/envmap.cpp"
#undef private

namespace drawlab {

namespace {
std::shared_ptr<Bitmap> g_harness_bitmap;
}

// The in-memory stand-in for the reference's file-backed "bitmap" texture.
class HarnessBitmapTexture : public Texture2D {
public:
    HarnessBitmapTexture(const PropertyList& props) : Texture2D(props) {}
    Color3f eval(const Point2f&) const { throw Exception("harness texture: eval"); }
    Color3f eval(const Point2f&, const Vector2f&, const Vector2f&) const {
        throw Exception("harness texture: eval");
    }
    bool isConstant() const { return false; }
    Vector3i getResolution() const {
        return Vector3i(g_harness_bitmap->getWidth(), g_harness_bitmap->getHeight(), 0);
    }
    std::shared_ptr<Bitmap> getBitmap(const Vector2i&) const { return g_harness_bitmap; }
    std::string toString() const { return "HarnessBitmapTexture[]"; }
};
REGISTER_CLASS(HarnessBitmapTexture, "bitmap");

}  // namespace drawlab

extern "C" {

// EnvironmentMap::activate on a height x width RGB float bitmap (row-major,
// row 0 first, as the reference's Bitmap holds it): the per-texel alias
// table (q, alias) and pdf.  Returns 0 on success.
int refx_env_tables(int32_t width, int32_t height, const float* rgb, float* q, uint32_t* alias, float* pdf) {
    using namespace drawlab;
    try {
        g_harness_bitmap = std::make_shared<Bitmap>(height, width);
        std::memcpy(g_harness_bitmap->getPtr(), rgb, sizeof(float) * 3 * (size_t)width * height);
        PropertyList props;
        props.setString("filename", "in-memory");
        EnvironmentMap env(props);
        env.activate();
        for (size_t i = 0; i < env.m_env_accel.size(); i++) {
            q[i] = env.m_env_accel[i].q;
            alias[i] = env.m_env_accel[i].alias;
            pdf[i] = env.m_env_accel[i].pdf;
        }
        g_harness_bitmap.reset();
        return 0;
    } catch (...) {
        return 1;
    }
}

// OpencvCamera(props) with `extrinsic` (row-major 4 x 4 world-to-camera
// matrix) and intrinsics, then getOptixCamera: the row-major inverse
// extrinsic and the eye.  Returns 0 on success.
int refx_opencv_setup(const float* extrinsic, float fx, float fy, float cx, float cy, float* inv_ext, float* eye) {
    using namespace drawlab;
    try {
        Matrix4f m;
        for (int i = 0; i < 16; i++) m.m[i / 4][i % 4] = extrinsic[i];
        PropertyList props;
        props.setTransform("extrinsic", Transform(m));
        props.setFloat("fx", fx);
        props.setFloat("fy", fy);
        props.setFloat("cx", cx);
        props.setFloat("cy", cy);
        std::unique_ptr<Camera> cam(static_cast<Camera*>(ObjectFactory::createInstance("opencv", props)));
        optix::Camera oc = cam->getOptixCamera();
        for (int i = 0; i < 16; i++) inv_ext[i] = oc.opencv_cam.invExt[i];
        eye[0] = oc.opencv_cam.eye.x;
        eye[1] = oc.opencv_cam.eye.y;
        eye[2] = oc.opencv_cam.eye.z;
        return 0;
    } catch (...) {
        return 1;
    }
}

}  // extern "C"
