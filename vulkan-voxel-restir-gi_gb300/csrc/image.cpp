// Image files of a frame: the headless replacement of the swapchain copy
// (interactive_rendering.rs:1625-1629).  BGRA8 frames are written as binary
// PPM or as PNG (8-bit RGB, zlib stream of stored deflate blocks: no
// compression library is needed and any PNG reader decodes it); float
// radiance as PFM.
#include <algorithm>
#include <array>
#include <cstdio>
#include <cstring>
#include <vector>

#include "vrg_internal.h"

namespace vrg {
namespace {

struct File {
    FILE *f = nullptr;
    explicit File(const char *path) : f(fopen(path, "wb")) {}
    ~File() {
        if (f) fclose(f);
    }
    bool put(const void *p, size_t n) { return fwrite(p, 1, n, f) == n; }
};

vrg_status open_check(File &fl, const char *path) {
    if (!fl.f) {
        set_error("cannot open %s for writing", path);
        return VRG_ERR_INVALID_ARGUMENT;
    }
    return VRG_OK;
}

uint32_t crc32_update(uint32_t crc, const uint8_t *p, size_t n) {
    // reflected CRC-32, polynomial 0xEDB88320 (the PNG / zlib CRC)
    static const std::array<uint32_t, 256> table = [] {
        std::array<uint32_t, 256> t{};
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t c = i;
            for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[i] = c;
        }
        return t;
    }();
    crc = ~crc;
    for (size_t i = 0; i < n; i++) crc = table[(crc ^ p[i]) & 0xFF] ^ (crc >> 8);
    return ~crc;
}

void put_be32(std::vector<uint8_t> &v, uint32_t x) {
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

bool png_chunk(File &fl, const char type[4], const std::vector<uint8_t> &data) {
    std::vector<uint8_t> head;
    put_be32(head, (uint32_t)data.size());
    head.insert(head.end(), type, type + 4);
    uint32_t crc = crc32_update(0, (const uint8_t *)type, 4);
    crc = crc32_update(crc, data.data(), data.size());
    std::vector<uint8_t> tail;
    put_be32(tail, crc);
    return fl.put(head.data(), head.size()) && (data.empty() || fl.put(data.data(), data.size())) &&
           fl.put(tail.data(), tail.size());
}

vrg_status check_args(const char *path, const void *px, uint32_t w, uint32_t h) {
    if (!path || !px || w == 0 || h == 0 || (uint64_t)w * h > (1ull << 31)) return VRG_ERR_INVALID_ARGUMENT;
    return VRG_OK;
}

}  // namespace
}  // namespace vrg

using namespace vrg;

extern "C" {

VRG_API vrg_status vrg_image_write_ppm(const char *path, const uint8_t *bgra8, uint32_t width, uint32_t height) {
    VRG_TRY(check_args(path, bgra8, width, height));
    File fl(path);
    VRG_TRY(open_check(fl, path));
    char head[64];
    const int n = snprintf(head, sizeof(head), "P6\n%u %u\n255\n", width, height);
    std::vector<uint8_t> rgb((size_t)width * height * 3);
    for (size_t i = 0; i < (size_t)width * height; i++) {
        rgb[3 * i] = bgra8[4 * i + 2];
        rgb[3 * i + 1] = bgra8[4 * i + 1];
        rgb[3 * i + 2] = bgra8[4 * i];
    }
    if (!fl.put(head, (size_t)n) || !fl.put(rgb.data(), rgb.size())) {
        set_error("write to %s failed", path);
        return VRG_ERR_INVALID_ARGUMENT;
    }
    return VRG_OK;
}

VRG_API vrg_status vrg_image_write_png(const char *path, const uint8_t *bgra8, uint32_t width, uint32_t height) {
    VRG_TRY(check_args(path, bgra8, width, height));
    File fl(path);
    VRG_TRY(open_check(fl, path));
    // raw scanlines: filter byte 0, then RGB
    const size_t row = 1 + (size_t)width * 3;
    std::vector<uint8_t> raw(row * height);
    for (uint32_t y = 0; y < height; y++) {
        uint8_t *d = raw.data() + row * y;
        d[0] = 0;
        const uint8_t *s = bgra8 + (size_t)4 * width * y;
        for (uint32_t x = 0; x < width; x++) {
            d[1 + 3 * x] = s[4 * x + 2];
            d[2 + 3 * x] = s[4 * x + 1];
            d[3 + 3 * x] = s[4 * x];
        }
    }
    // zlib stream: header, stored blocks of at most 65535 bytes, Adler-32
    std::vector<uint8_t> z = {0x78, 0x01};
    size_t off = 0;
    do {
        const size_t n = std::min<size_t>(65535, raw.size() - off);
        const bool last = off + n == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)(n & 0xFF));
        z.push_back((uint8_t)(n >> 8));
        z.push_back((uint8_t)(~n & 0xFF));
        z.push_back((uint8_t)((~n >> 8) & 0xFF));
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + n);
        off += n;
    } while (off < raw.size());
    uint32_t a = 1, b = 0;
    for (uint8_t c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    put_be32(z, (b << 16) | a);
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, width);
    put_be32(ihdr, height);
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});  // 8-bit, truecolour, deflate, filter 0, no interlace
    if (!fl.put(sig, 8) || !png_chunk(fl, "IHDR", ihdr) || !png_chunk(fl, "IDAT", z) ||
        !png_chunk(fl, "IEND", {})) {
        set_error("write to %s failed", path);
        return VRG_ERR_INVALID_ARGUMENT;
    }
    return VRG_OK;
}

VRG_API vrg_status vrg_image_write_pfm(const char *path, const float *rgb, uint32_t width, uint32_t height) {
    VRG_TRY(check_args(path, rgb, width, height));
    File fl(path);
    VRG_TRY(open_check(fl, path));
    char head[64];
    const int n = snprintf(head, sizeof(head), "PF\n%u %u\n-1.0\n", width, height);  // -1: little-endian
    if (!fl.put(head, (size_t)n)) {
        set_error("write to %s failed", path);
        return VRG_ERR_INVALID_ARGUMENT;
    }
    std::vector<uint8_t> rowb((size_t)width * 12);
    for (uint32_t y = 0; y < height; y++) {  // PFM stores the bottom row first
        const float *src = rgb + (size_t)3 * width * (height - 1 - y);
        for (size_t i = 0; i < (size_t)3 * width; i++) {
            uint32_t bits;
            memcpy(&bits, src + i, 4);
            rowb[4 * i] = (uint8_t)bits;
            rowb[4 * i + 1] = (uint8_t)(bits >> 8);
            rowb[4 * i + 2] = (uint8_t)(bits >> 16);
            rowb[4 * i + 3] = (uint8_t)(bits >> 24);
        }
        if (!fl.put(rowb.data(), rowb.size())) {
            set_error("write to %s failed", path);
            return VRG_ERR_INVALID_ARGUMENT;
        }
    }
    return VRG_OK;
}

}  // extern "C"
