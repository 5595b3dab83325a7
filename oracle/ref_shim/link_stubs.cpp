// Link-time stand-ins for reference symbols whose definitions live in files the
// harness does not compile (src/core/bitmap/bitmap.cpp needs OpenEXR/stb;
// src/optix/host/cuda_texture.cpp needs the CUDA runtime).  block.cpp and
// texture.cpp reference them from code the harness never calls
// (ImageBlock::toBitmap/fromBitmap, texture upload); each aborts if reached.
#include <cstdlib>
#include "core/bitmap/bitmap.h"
#include "optix/host/cuda_texture.h"

namespace drawlab {
Bitmap::Bitmap(int, int) { std::abort(); }
Bitmap::~Bitmap() {}
void Bitmap::setPixel(int, int, Color3f) { std::abort(); }
Color3f Bitmap::getPixel(int, int) const { std::abort(); }
}  // namespace drawlab

namespace optix {
const cudaTextureObject_t CUDATexture::getObject() const { std::abort(); }
}  // namespace optix
