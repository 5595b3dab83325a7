// Host stand-in for the OptiX device API, used only when the reference's
// OptiX shaders are compiled as host C++ (test infrastructure:
// oracle/ref_optix.cpp).  The ray and hit queries return what the harness
// stored in refshim::g_optix before it calls a shader function; optixTrace
// is never reached by the harness.
#pragma once
#include <vector_types.h>

typedef unsigned long long OptixTraversableHandle;
typedef unsigned int OptixVisibilityMask;
enum OptixRayFlags { OPTIX_RAY_FLAG_NONE = 0, OPTIX_RAY_FLAG_TERMINATE_ON_FIRST_HIT = 4 };
#define OPTIX_SBT_RECORD_HEADER_SIZE 32
#define OPTIX_SBT_RECORD_ALIGNMENT 16

namespace refshim {
struct OptixState {
    float3 ray_o, ray_d;
    float tmax;
    unsigned int payload0, payload1;
    const void* sbt;
    int prim;
    float2 bary;
};
extern OptixState g_optix;
}  // namespace refshim

inline float3 optixGetWorldRayDirection() { return refshim::g_optix.ray_d; }
inline float3 optixGetWorldRayOrigin() { return refshim::g_optix.ray_o; }
inline float optixGetRayTmax() { return refshim::g_optix.tmax; }
inline unsigned int optixGetPayload_0() { return refshim::g_optix.payload0; }
inline unsigned int optixGetPayload_1() { return refshim::g_optix.payload1; }
inline void optixSetPayload_0(unsigned int v) { refshim::g_optix.payload0 = v; }
inline const void* optixGetSbtDataPointer() { return refshim::g_optix.sbt; }
inline int optixGetPrimitiveIndex() { return refshim::g_optix.prim; }
inline float2 optixGetTriangleBarycentrics() { return refshim::g_optix.bary; }
template <typename... A>
inline void optixTrace(A&&...) {}
