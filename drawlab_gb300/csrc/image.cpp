// Image output: dl_image_write (PNG, OpenEXR, PFM) for rendered RGB images.
// Host code only; no CUDA.
//
// PNG follows Bitmap::savePNG (src/core/bitmap/bitmap.cpp:190-214): each
// linear value goes through Color3f::toSRGB (include/core/bitmap/color.h:
// 76-87), is scaled by 255, clamped to [0, 255] and truncated to 8 bits.
// The file holds one IDAT chunk whose zlib stream uses stored (uncompressed)
// deflate blocks: valid PNG without a compression library.
//
// OpenEXR follows Bitmap::saveEXR (bitmap.cpp:157-188): float R, G, B
// channels, scanline file, here without compression (one scanline per
// chunk, offset table, channels in alphabetical order as the format asks).
//
// PFM: "PF", little-endian floats, rows bottom to top.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"
#include "scene.h"

namespace dl {
namespace {

struct File {
    FILE* f = nullptr;
    explicit File(const char* path) : f(std::fopen(path, "wb")) {}
    ~File() {
        if (f) std::fclose(f);
    }
    void write(const void* p, size_t n) {
        if (n && std::fwrite(p, 1, n, f) != n) throw Error(DL_ERR_IO, "write failed");
    }
};

// ---------------------------------------------------------------- PNG
struct CrcTable {
    uint32_t t[256];
    CrcTable() {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t c = i;
            for (int k = 0; k < 8; k++) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[i] = c;
        }
    }
};

uint32_t crc32_update(uint32_t crc, const uint8_t* p, size_t n) {  // the CRC of ISO 3309, as PNG uses
    static const CrcTable table;
    for (size_t i = 0; i < n; i++) crc = table.t[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return crc;
}

void put_be32(std::vector<uint8_t>& v, uint32_t x) {
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

void png_chunk(File& out, const char* type, const std::vector<uint8_t>& data) {
    std::vector<uint8_t> head;
    put_be32(head, (uint32_t)data.size());
    out.write(head.data(), 4);
    uint32_t crc = crc32_update(0xFFFFFFFFu, reinterpret_cast<const uint8_t*>(type), 4);
    crc = crc32_update(crc, data.data(), data.size());
    out.write(type, 4);
    out.write(data.data(), data.size());
    std::vector<uint8_t> tail;
    put_be32(tail, crc ^ 0xFFFFFFFFu);
    out.write(tail.data(), 4);
}

// Color3f::toSRGB, per channel
float to_srgb(float v) {
    if (v <= 0.0031308f) return 12.92f * v;
    return (1.0f + 0.055f) * std::pow(v, 1.0f / 2.4f) - 0.055f;
}

uint8_t to_byte(float v) {
    float x = 255.f * to_srgb(v);
    if (!(x == x)) return 0;                        // NaN: 0
    x = x < 0.f ? 0.f : (x > 255.f ? 255.f : x);  // clamp(255 v, 0, 255)
    return (uint8_t)x;
}

void write_png(const char* path, int w, int h, const float* rgb) {
    // raw scanlines: filter type 0, then RGB bytes
    std::vector<uint8_t> raw;
    raw.reserve((size_t)h * (3 * (size_t)w + 1));
    for (int y = 0; y < h; y++) {
        raw.push_back(0);
        for (int x = 0; x < 3 * w; x++) raw.push_back(to_byte(rgb[(size_t)y * 3 * w + x]));
    }
    // zlib stream of stored deflate blocks (RFC 1950 / 1951)
    std::vector<uint8_t> z;
    z.push_back(0x78);
    z.push_back(0x01);
    size_t pos = 0;
    do {
        const size_t n = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + n == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)(n & 0xFF));
        z.push_back((uint8_t)(n >> 8));
        z.push_back((uint8_t)(~n & 0xFF));
        z.push_back((uint8_t)((~n >> 8) & 0xFF));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
        pos += n;
    } while (pos < raw.size());
    uint32_t a = 1, b = 0;  // Adler-32
    for (uint8_t c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    put_be32(z, (b << 16) | a);
    File out(path);
    if (!out.f) throw Error(DL_ERR_IO, std::string("cannot open ") + path);
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    out.write(sig, 8);
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, (uint32_t)w);
    put_be32(ihdr, (uint32_t)h);
    ihdr.push_back(8);  // bit depth
    ihdr.push_back(2);  // colour type: RGB
    ihdr.push_back(0);  // deflate
    ihdr.push_back(0);  // adaptive filtering
    ihdr.push_back(0);  // no interlace
    png_chunk(out, "IHDR", ihdr);
    png_chunk(out, "IDAT", z);
    png_chunk(out, "IEND", {});
}

// ------------------------------------------------------------- OpenEXR
void put_le32(std::vector<uint8_t>& v, uint32_t x) {
    for (int k = 0; k < 4; k++) v.push_back((uint8_t)(x >> (8 * k)));
}
void put_le64(std::vector<uint8_t>& v, uint64_t x) {
    for (int k = 0; k < 8; k++) v.push_back((uint8_t)(x >> (8 * k)));
}
void put_f32(std::vector<uint8_t>& v, float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    put_le32(v, u);
}
void put_str(std::vector<uint8_t>& v, const char* s) {
    v.insert(v.end(), s, s + std::strlen(s) + 1);
}
void attr(std::vector<uint8_t>& h, const char* name, const char* type, const std::vector<uint8_t>& value) {
    put_str(h, name);
    put_str(h, type);
    put_le32(h, (uint32_t)value.size());
    h.insert(h.end(), value.begin(), value.end());
}

void write_exr(const char* path, int w, int h, const float* rgb) {
    std::vector<uint8_t> hd;
    put_le32(hd, 20000630u);  // magic
    put_le32(hd, 2u);         // version 2, single-part scanline
    std::vector<uint8_t> v;
    for (const char* ch : {"B", "G", "R"}) {
        put_str(v, ch);
        put_le32(v, 2u);  // FLOAT
        v.push_back(0);   // pLinear
        v.push_back(0);
        v.push_back(0);
        v.push_back(0);
        put_le32(v, 1u);  // x sampling
        put_le32(v, 1u);  // y sampling
    }
    v.push_back(0);
    attr(hd, "channels", "chlist", v);
    attr(hd, "compression", "compression", {0});
    v.clear();
    put_le32(v, 0);
    put_le32(v, 0);
    put_le32(v, (uint32_t)(w - 1));
    put_le32(v, (uint32_t)(h - 1));
    attr(hd, "dataWindow", "box2i", v);
    attr(hd, "displayWindow", "box2i", v);
    attr(hd, "lineOrder", "lineOrder", {0});
    v.clear();
    put_f32(v, 1.f);
    attr(hd, "pixelAspectRatio", "float", v);
    v.clear();
    put_f32(v, 0.f);
    put_f32(v, 0.f);
    attr(hd, "screenWindowCenter", "v2f", v);
    v.clear();
    put_f32(v, 1.f);
    attr(hd, "screenWindowWidth", "float", v);
    hd.push_back(0);  // end of header
    const uint64_t line_bytes = (uint64_t)w * 3 * 4;
    const uint64_t chunk = 8 + line_bytes;
    const uint64_t first = hd.size() + 8 * (uint64_t)h;
    for (int y = 0; y < h; y++) put_le64(hd, first + (uint64_t)y * chunk);
    File out(path);
    if (!out.f) throw Error(DL_ERR_IO, std::string("cannot open ") + path);
    out.write(hd.data(), hd.size());
    std::vector<uint8_t> line;
    for (int y = 0; y < h; y++) {
        line.clear();
        put_le32(line, (uint32_t)y);
        put_le32(line, (uint32_t)line_bytes);
        for (int c = 2; c >= 0; c--)  // B, G, R
            for (int x = 0; x < w; x++) put_f32(line, rgb[((size_t)y * w + x) * 3 + c]);
        out.write(line.data(), line.size());
    }
}

// ----------------------------------------------------------------- PFM
void write_pfm(const char* path, int w, int h, const float* rgb) {
    File out(path);
    if (!out.f) throw Error(DL_ERR_IO, std::string("cannot open ") + path);
    const std::string head = "PF\n" + std::to_string(w) + " " + std::to_string(h) + "\n-1.0\n";
    out.write(head.data(), head.size());
    std::vector<uint8_t> row;
    for (int y = h - 1; y >= 0; y--) {
        row.clear();
        for (int x = 0; x < 3 * w; x++) put_f32(row, rgb[(size_t)y * 3 * w + x]);
        out.write(row.data(), row.size());
    }
}

}  // namespace
}  // namespace dl

namespace dl {
void write_image(const char* path, int width, int height, const float* rgb, int format) {
    if (!path || !rgb || width <= 0 || height <= 0 || width > 65536 || height > 65536)
        throw Error(DL_ERR_INVALID_ARG, "bad image arguments");
    switch (format) {
        case DL_IMAGE_PNG: write_png(path, width, height, rgb); break;
        case DL_IMAGE_EXR: write_exr(path, width, height, rgb); break;
        case DL_IMAGE_PFM: write_pfm(path, width, height, rgb); break;
        default: throw Error(DL_ERR_INVALID_ARG, "unknown image format");
    }
}
}  // namespace dl
