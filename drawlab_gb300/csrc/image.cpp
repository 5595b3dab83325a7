// Image output: dl_image_write (PNG, OpenEXR, PFM) for rendered RGB images;
// image input: dl_image_read / read_image (PNG, PFM) for textures and
// envmaps.  Host code only; no CUDA.
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
//
// PNG input: 8-bit grey, grey + alpha, RGB, RGBA and palette images without
// interlacing, decoded with the inflate algorithm of RFC 1951 (stored,
// fixed-Huffman and dynamic-Huffman blocks; canonical Huffman codes decoded
// length by length) and the five scanline filters of the PNG specification.
// Values are the bytes / 255 (the reference uploads 8-bit textures as
// linear RGBA8, src/tracer/texture/bitmap.cpp:66-77); alpha is dropped.
#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
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


// --------------------------------------------------------------- inflate
struct Bits {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    int get(int k) {  // k <= 24 bits, least significant first
        while (cnt < k) {
            if (pos >= n) throw Error(DL_ERR_PARSE, "truncated deflate stream");
            buf |= (uint32_t)p[pos++] << cnt;
            cnt += 8;
        }
        const int v = (int)(buf & ((1u << k) - 1u));
        buf >>= k;
        cnt -= k;
        return v;
    }
};

struct Huffman {
    int count[16] = {0};  // codes per length
    std::vector<int> sym;  // symbols ordered by (length, value)
    void build(const int* lengths, int n) {
        std::fill(count, count + 16, 0);
        for (int i = 0; i < n; i++) count[lengths[i]]++;
        count[0] = 0;
        int offs[16];
        offs[1] = 0;
        for (int l = 1; l < 15; l++) offs[l + 1] = offs[l] + count[l];
        sym.assign(n, 0);
        for (int i = 0; i < n; i++)
            if (lengths[i]) sym[offs[lengths[i]]++] = i;
    }
    int decode(Bits& b) const {
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; l++) {
            code |= b.get(1);
            const int c = count[l];
            if (code - first < c) return sym[index + code - first];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        throw Error(DL_ERR_PARSE, "bad Huffman code");
    }
};

// RFC 1951 3.2.5: base lengths / distances and their extra bits
const int kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                          35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const int kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const int kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193,
                           257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const int kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

void inflate_codes(Bits& b, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out, size_t limit) {
    for (;;) {
        const int s = lit.decode(b);
        if (s < 256) {
            out.push_back((uint8_t)s);
        } else if (s == 256) {
            return;
        } else {
            const int li = s - 257;
            if (li >= 29) throw Error(DL_ERR_PARSE, "bad length code");
            const int len = kLenBase[li] + b.get(kLenExtra[li]);
            const int di = dist.decode(b);
            if (di >= 30) throw Error(DL_ERR_PARSE, "bad distance code");
            const size_t d = (size_t)(kDistBase[di] + b.get(kDistExtra[di]));
            if (d > out.size()) throw Error(DL_ERR_PARSE, "distance beyond the output");
            for (int k = 0; k < len; k++) out.push_back(out[out.size() - d]);
        }
        if (out.size() > limit) throw Error(DL_ERR_PARSE, "inflated data larger than the image");
    }
}

std::vector<uint8_t> inflate(const uint8_t* p, size_t n, size_t limit) {
    Bits b{p, n};
    std::vector<uint8_t> out;
    int last = 0;
    while (!last) {
        last = b.get(1);
        const int type = b.get(2);
        if (type == 0) {  // stored
            b.buf = 0;
            b.cnt = 0;
            if (b.pos + 4 > n) throw Error(DL_ERR_PARSE, "truncated stored block");
            const size_t len = p[b.pos] | (p[b.pos + 1] << 8);
            const size_t nlen = p[b.pos + 2] | (p[b.pos + 3] << 8);
            if ((len ^ 0xFFFFu) != nlen) throw Error(DL_ERR_PARSE, "bad stored block length");
            b.pos += 4;
            if (b.pos + len > n) throw Error(DL_ERR_PARSE, "truncated stored block");
            out.insert(out.end(), p + b.pos, p + b.pos + len);
            b.pos += len;
        } else if (type == 1) {  // fixed Huffman codes (RFC 1951 3.2.6)
            static Huffman lit, dist;
            static bool init = false;
            if (!init) {
                int l[288];
                for (int i = 0; i < 288; i++) l[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
                lit.build(l, 288);
                int d[30];
                for (int i = 0; i < 30; i++) d[i] = 5;
                dist.build(d, 30);
                init = true;
            }
            inflate_codes(b, lit, dist, out, limit);
        } else if (type == 2) {  // dynamic Huffman codes (RFC 1951 3.2.7)
            const int hlit = b.get(5) + 257, hdist = b.get(5) + 1, hclen = b.get(4) + 4;
            static const int order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            int cl[19] = {0};
            for (int i = 0; i < hclen; i++) cl[order[i]] = b.get(3);
            Huffman clh;
            clh.build(cl, 19);
            int lens[320] = {0};
            int k = 0;
            while (k < hlit + hdist) {
                const int s = clh.decode(b);
                if (s < 16) {
                    lens[k++] = s;
                } else {
                    int rep = 0, val = 0;
                    if (s == 16) {
                        if (k == 0) throw Error(DL_ERR_PARSE, "repeat without a length");
                        val = lens[k - 1];
                        rep = 3 + b.get(2);
                    } else if (s == 17) {
                        rep = 3 + b.get(3);
                    } else {
                        rep = 11 + b.get(7);
                    }
                    if (k + rep > hlit + hdist) throw Error(DL_ERR_PARSE, "too many code lengths");
                    while (rep--) lens[k++] = val;
                }
            }
            Huffman lit, dist;
            lit.build(lens, hlit);
            dist.build(lens + hlit, hdist);
            inflate_codes(b, lit, dist, out, limit);
        } else {
            throw Error(DL_ERR_PARSE, "bad deflate block type");
        }
        if (out.size() > limit) throw Error(DL_ERR_PARSE, "inflated data larger than the image");
    }
    return out;
}

uint32_t be32(const uint8_t* p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

std::vector<uint8_t> read_file(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) throw Error(DL_ERR_IO, "cannot open image \"" + path + "\"");
    std::vector<uint8_t> d;
    uint8_t buf[65536];
    size_t k;
    while ((k = std::fread(buf, 1, sizeof(buf), f)) > 0) d.insert(d.end(), buf, buf + k);
    std::fclose(f);
    return d;
}

// PNG -> RGB floats (bytes / 255), row 0 = the image's top row.
std::vector<float> read_png(const std::string& path, int& w, int& h) {
    const std::vector<uint8_t> d = read_file(path);
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    if (d.size() < 8 || std::memcmp(d.data(), sig, 8) != 0) throw Error(DL_ERR_PARSE, "\"" + path + "\": not a PNG image");
    size_t pos = 8;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, plte;
    w = h = 0;
    while (pos + 12 <= d.size()) {
        const uint32_t n = be32(&d[pos]);
        if (pos + 12 + (size_t)n > d.size()) throw Error(DL_ERR_PARSE, "\"" + path + "\": truncated chunk");
        const char* t = reinterpret_cast<const char*>(&d[pos + 4]);
        const uint8_t* body = &d[pos + 8];
        if (std::memcmp(t, "IHDR", 4) == 0 && n >= 13) {
            w = (int)be32(body);
            h = (int)be32(body + 4);
            depth = body[8];
            ctype = body[9];
            interlace = body[12];
        } else if (std::memcmp(t, "PLTE", 4) == 0) {
            plte.assign(body, body + n);
        } else if (std::memcmp(t, "IDAT", 4) == 0) {
            idat.insert(idat.end(), body, body + n);
        } else if (std::memcmp(t, "IEND", 4) == 0) {
            break;
        }
        pos += 12 + n;
    }
    if (w <= 0 || h <= 0 || (int64_t)w * h > ((int64_t)1 << 26)) throw Error(DL_ERR_PARSE, "\"" + path + "\": bad PNG size");
    if (depth != 8 || interlace != 0 || !(ctype == 0 || ctype == 2 || ctype == 3 || ctype == 4 || ctype == 6))
        throw Error(DL_ERR_UNSUPPORTED, "\"" + path + "\": only 8-bit, non-interlaced PNG images are supported");
    if (ctype == 3 && plte.size() < 3) throw Error(DL_ERR_PARSE, "\"" + path + "\": palette missing");
    if (idat.size() < 2 || (idat[0] & 0x0F) != 8) throw Error(DL_ERR_PARSE, "\"" + path + "\": bad zlib stream");
    const int ch = ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 3 ? 1 : ctype == 4 ? 2 : 4;
    const size_t stride = (size_t)w * ch;
    const std::vector<uint8_t> raw = inflate(idat.data() + 2, idat.size() - 2, (stride + 1) * (size_t)h);
    if (raw.size() < (stride + 1) * (size_t)h) throw Error(DL_ERR_PARSE, "\"" + path + "\": short image data");
    std::vector<uint8_t> img(stride * (size_t)h);
    for (int y = 0; y < h; y++) {
        const uint8_t filter = raw[(size_t)y * (stride + 1)];
        const uint8_t* src = &raw[(size_t)y * (stride + 1) + 1];
        uint8_t* cur = &img[(size_t)y * stride];
        const uint8_t* prev = y > 0 ? &img[(size_t)(y - 1) * stride] : nullptr;
        for (size_t i = 0; i < stride; i++) {
            const int a = i >= (size_t)ch ? cur[i - ch] : 0;
            const int b = prev ? prev[i] : 0;
            const int c = (prev && i >= (size_t)ch) ? prev[i - ch] : 0;
            int v = src[i];
            switch (filter) {
                case 0: break;
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) >> 1; break;
                case 4: {
                    const int p0 = a + b - c, pa = std::abs(p0 - a), pb = std::abs(p0 - b), pc = std::abs(p0 - c);
                    v += (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
                    break;
                }
                default: throw Error(DL_ERR_PARSE, "\"" + path + "\": bad scanline filter");
            }
            cur[i] = (uint8_t)v;
        }
    }
    std::vector<float> rgb((size_t)w * h * 3);
    for (size_t i = 0; i < (size_t)w * h; i++) {
        uint8_t r, g, bl;
        if (ctype == 3) {
            const size_t k = 3 * (size_t)img[i];
            if (k + 2 >= plte.size()) throw Error(DL_ERR_PARSE, "\"" + path + "\": palette index out of range");
            r = plte[k];
            g = plte[k + 1];
            bl = plte[k + 2];
        } else if (ch <= 2) {
            r = g = bl = img[i * ch];
        } else {
            r = img[i * ch];
            g = img[i * ch + 1];
            bl = img[i * ch + 2];
        }
        rgb[3 * i] = r / 255.f;
        rgb[3 * i + 1] = g / 255.f;
        rgb[3 * i + 2] = bl / 255.f;
    }
    return rgb;
}

}  // namespace
}  // namespace dl

namespace dl {
// Portable float map (PF: RGB, Pf: grey), rows stored bottom to top, scale
// sign = byte order.  Returns rows top to bottom, RGB.  The reference reads
// envmaps through its Bitmap class (EXR via OpenEXR, LDR/HDR via stb_image,
// src/core/bitmap/bitmap.cpp:30-140); this library reads PFM.
std::vector<float> load_pfm(const std::string& path, int& w, int& h) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw Error(DL_ERR_IO, "cannot open image \"" + path + "\"");
    std::string magic;
    double scale = 0;
    in >> magic >> w >> h >> scale;
    if (!in || (magic != "PF" && magic != "Pf") || w <= 0 || h <= 0 || (int64_t)w * h > ((int64_t)1 << 26) ||
        scale == 0)
        throw Error(DL_ERR_PARSE, "\"" + path + "\": not a PFM image");
    in.get();  // the single whitespace byte before the raster
    const int ch = magic == "PF" ? 3 : 1;
    std::vector<float> raw((size_t)w * h * ch);
    in.read(reinterpret_cast<char*>(raw.data()), (std::streamsize)(raw.size() * 4));
    if (!in) throw Error(DL_ERR_PARSE, "\"" + path + "\": truncated PFM raster");
    const uint16_t probe = 1;
    const bool host_le = *reinterpret_cast<const uint8_t*>(&probe) == 1;
    if ((scale < 0) != host_le) {
        for (float& v : raw) {
            uint8_t* b = reinterpret_cast<uint8_t*>(&v);
            std::swap(b[0], b[3]);
            std::swap(b[1], b[2]);
        }
    }
    std::vector<float> rgb((size_t)w * h * 3);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
            for (int c = 0; c < 3; c++)
                rgb[3 * ((size_t)y * w + x) + c] = raw[ch * ((size_t)(h - 1 - y) * w + x) + (ch == 3 ? c : 0)];
    return rgb;
}

std::vector<float> read_image(const std::string& path, int& w, int& h, bool& is_float) {
    const size_t dot = path.find_last_of('.');
    std::string ext = dot == std::string::npos ? "" : path.substr(dot + 1);
    for (char& c : ext) c = (char)std::tolower((unsigned char)c);
    if (ext == "pfm") {
        is_float = true;
        return load_pfm(path, w, h);
    }
    if (ext == "png") {
        is_float = false;
        return read_png(path, w, h);
    }
    throw Error(DL_ERR_UNSUPPORTED, "image \"" + path + "\": only PNG and PFM images can be read");
}

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
