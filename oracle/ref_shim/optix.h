// Stand-in for the absent OptiX SDK header: opaque handle types only, so that
// the reference's plugin headers (which declare OptiX packing methods) compile.
// Nothing here is called by the CPU path.
#pragma once
#include <cuda.h>
typedef struct OptixDeviceContext_t* OptixDeviceContext;
typedef struct OptixModule_t* OptixModule;
typedef struct OptixProgramGroup_t* OptixProgramGroup;
typedef struct OptixPipeline_t* OptixPipeline;
typedef unsigned long long OptixTraversableHandle;
struct OptixPipelineCompileOptions { int unused; };
struct OptixPipelineLinkOptions { int unused; };
struct OptixModuleCompileOptions { int unused; };
struct OptixShaderBindingTable { int unused; };
struct OptixBuildInput { int unused; };
typedef int OptixResult;
#define OPTIX_SBT_RECORD_HEADER_SIZE 32
#define OPTIX_SBT_RECORD_ALIGNMENT 16
inline const char* optixGetErrorName(OptixResult) { return "optix-absent"; }
inline const char* optixGetErrorString(OptixResult) { return "optix-absent"; }
