// Link-time stand-ins for reference symbols whose definitions live in files the
// harness does not compile (src/core/bitmap/bitmap.cpp needs OpenEXR/stb;
// src/optix/host/cuda_texture.cpp needs the CUDA runtime).  The in-memory
// Bitmap(height, width) holds a zeroed RGB float image (the envmap harness
// fills it); the texture upload is never called and aborts if reached.
#include <cstdlib>
#include "core/bitmap/bitmap.h"
#include "optix/host/cuda_texture.h"

namespace drawlab {
Bitmap::Bitmap(int height, int width)
    : m_width(width), m_height(height), m_data((size_t)width * height * 3, 0.0f), m_format(FLOAT3) {}
Bitmap::~Bitmap() {}
void Bitmap::setPixel(int row, int col, Color3f c) {
    float* p = &m_data[3 * ((size_t)row * m_width + col)];
    p[0] = c[0];
    p[1] = c[1];
    p[2] = c[2];
}
Color3f Bitmap::getPixel(int row, int col) const {
    const float* p = &m_data[3 * ((size_t)row * m_width + col)];
    return Color3f(p[0], p[1], p[2]);
}
}  // namespace drawlab

namespace optix {
const cudaTextureObject_t CUDATexture::getObject() const { std::abort(); }
}  // namespace optix

// CUDABuffer (include/optix/host/cuda_buffer.h) reaches the CUDA runtime
// from EnvironmentMap::getOptixLight, which the harness never calls.
extern "C" {
cudaError_t cudaMalloc(void**, size_t) { std::abort(); }
cudaError_t cudaMemcpy(void*, const void*, size_t, cudaMemcpyKind) { std::abort(); }
const char* cudaGetErrorString(cudaError_t) { std::abort(); }
}
