// Host stand-in for <cuda_runtime.h>, used only when the reference's OptiX
// device headers and shaders are compiled as host C++ by g++ (test
// infrastructure: oracle/ref_optix.cpp).  It provides CUDA's vector types
// (the toolkit's own vector_types.h / vector_functions.h), the integer
// min/max overloads that device code gets from the CUDA math headers, and a
// host model of tex2D<float4> for the reference's textures (normalized
// coordinates, linear filtering, wrap addressing, cuda_texture.cpp:57-84).
#pragma once

#include <vector_functions.h>
#include <vector_types.h>

#include <cmath>
#include <cstdint>
#include <cstdio>

typedef unsigned long long cudaTextureObject_t;

inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline unsigned int min(unsigned int a, unsigned int b) { return a < b ? a : b; }
inline unsigned int max(unsigned int a, unsigned int b) { return a > b ? a : b; }
inline long long min(long long a, long long b) { return a < b ? a : b; }
inline long long max(long long a, long long b) { return a > b ? a : b; }
inline unsigned long long min(unsigned long long a, unsigned long long b) { return a < b ? a : b; }
inline unsigned long long max(unsigned long long a, unsigned long long b) { return a > b ? a : b; }
using std::fmax;
using std::fmin;
using std::isnan;

// bit casts of the CUDA device intrinsics
inline int __float_as_int(float f) {
    int i;
    __builtin_memcpy(&i, &f, sizeof(i));
    return i;
}
inline float __int_as_float(int i) {
    float f;
    __builtin_memcpy(&f, &i, sizeof(f));
    return f;
}

namespace refshim {
// One texture object of the host model: RGBA texels, row 0 first, already
// in the read mode's value range.
struct HostTexture {
    int width = 0, height = 0;
    const float4* texels = nullptr;
};
// Registry indexed by cudaTextureObject_t - 1 (0 is "no texture").
HostTexture* texture_slot(cudaTextureObject_t obj);
// Filter weights of the texture unit: CUDA stores them in 9-bit fixed point
// with 8 fractional bits (CUDA C Programming Guide, "Linear Filtering").
// When `quantised` is false the host model keeps fp32 weights instead.
extern bool g_quantised_weights;
float4 tex2d_linear_wrap(const HostTexture& t, float u, float v);
}  // namespace refshim

template <class T>
T tex2D(cudaTextureObject_t obj, float x, float y);

template <>
inline float4 tex2D<float4>(cudaTextureObject_t obj, float x, float y) {
    return refshim::tex2d_linear_wrap(*refshim::texture_slot(obj), x, y);
}
