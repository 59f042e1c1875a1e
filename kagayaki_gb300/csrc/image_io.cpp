// image_io.cpp - tone mapping and PNG output (replaces save_png,
// FileIO/IO_save_png.cuh:7-56).  The PNG encoder writes stored (uncompressed)
// deflate blocks, so the library needs no zlib.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <mutex>
#include <vector>

#include "kgk_scene.h"

using namespace kgk;

namespace {

uint32_t crc_table[256];
bool crc_ready = false;

void crc_init() {
    for (uint32_t n = 0; n < 256; ++n) {
        uint32_t c = n;
        for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xedb88320u ^ (c >> 1) : c >> 1;
        crc_table[n] = c;
    }
    crc_ready = true;
}

uint32_t crc32(const uint8_t *p, size_t n, uint32_t c = 0xffffffffu) {
    for (size_t i = 0; i < n; ++i) c = crc_table[(c ^ p[i]) & 0xff] ^ (c >> 8);
    return c;
}

void put32(std::vector<uint8_t> &v, uint32_t x) {
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

void chunk(std::vector<uint8_t> &out, const char *type, const std::vector<uint8_t> &data) {
    put32(out, (uint32_t)data.size());
    size_t start = out.size();
    out.insert(out.end(), type, type + 4);
    out.insert(out.end(), data.begin(), data.end());
    put32(out, crc32(&out[start], out.size() - start) ^ 0xffffffffu);
}

inline uint8_t tone(float x) { return kgk::tone_host(x); }

}  // namespace

namespace kgk {

// gamma 1/2.2 -> clamp [0,1] -> x255 truncated (IO_save_png.cuh:26,7,47-52);
// a NaN (also powf of a negative number) gives 0 instead of the reference's
// undefined float-to-char conversion.
uint8_t tone_host(float x) {
    float g = powf(x, 1 / 2.2f);
    if (g != g) return 0;
    g = g < 0.0f ? 0.0f : (g > 1.0f ? 1.0f : g);
    return (uint8_t)(g * 255);
}

const float *tone_thresholds() {
    static float t[255];
    static std::once_flag once;
    std::call_once(once, []() {
        // floats >= 0 are ordered like their bit patterns: binary search over
        // [+0, +inf] for the first pattern whose byte reaches k
        for (int k = 1; k <= 255; ++k) {
            uint32_t lo = 0u, hi = 0x7f800000u;  // tone_host(+inf) = 255 >= k
            while (lo < hi) {
                const uint32_t mid = lo + (hi - lo) / 2;
                float x;
                memcpy(&x, &mid, 4);
                if (tone_host(x) >= k) hi = mid;
                else lo = mid + 1;
            }
            memcpy(&t[k - 1], &lo, 4);
        }
    });
    return t;
}

}  // namespace kgk

extern "C" {

kgk_status kgk_tonemap_rgba8(const kgk_vec *img, int32_t w, int32_t h, uint8_t *out) {
    KGK_GUARD_BEGIN
    if (!img || !out) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_tonemap_rgba8: NULL buffer");
    if (w <= 0 || h <= 0) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_tonemap_rgba8: empty image");
    const size_t npx = (size_t)w * h;
    const kgk_vec *src = img;
    if (is_device_ptr(img)) {
        // on the device; the bytes go to `out` (device or host)
        uchar4 *dout = reinterpret_cast<uchar4 *>(out);
        const bool od = is_device_ptr(out);
        if (!od) KGK_CUDA(cudaMalloc(reinterpret_cast<void **>(&dout), npx * sizeof(uchar4)));
        kgk_status st = tonemap_device(reinterpret_cast<const float4 *>(img), npx, dout, nullptr);
        if (st == KGK_OK && !od) {
            const cudaError_t e = cudaMemcpy(out, dout, npx * sizeof(uchar4), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) st = cuda_fail(e, "kgk_tonemap_rgba8 copy");
        }
        if (st == KGK_OK) {
            const cudaError_t e = cudaDeviceSynchronize();
            if (e != cudaSuccess) st = cuda_fail(e, "kgk_tonemap_rgba8");
        }
        if (!od) cudaFree(dout);
        return st;
    }
    for (size_t i = 0; i < npx; ++i) {
        out[4 * i] = tone(src[i].x);
        out[4 * i + 1] = tone(src[i].y);
        out[4 * i + 2] = tone(src[i].z);
        out[4 * i + 3] = 255;
    }
    return KGK_OK;
    KGK_GUARD_END
}

kgk_status kgk_save_png(const kgk_vec *img, int32_t w, int32_t h, const char *path) {
    KGK_GUARD_BEGIN
    if (!path) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_save_png: path == NULL");
    if (w <= 0 || h <= 0) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_save_png: empty image");
    std::vector<uint8_t> rgba((size_t)w * h * 4);
    KGK_TRY(kgk_tonemap_rgba8(img, w, h, rgba.data()));
    if (!crc_ready) crc_init();
    std::vector<uint8_t> raw;
    raw.reserve((size_t)h * (4 * (size_t)w + 1));
    for (int y = 0; y < h; ++y) {
        raw.push_back(0);  // filter: none
        raw.insert(raw.end(), rgba.begin() + (size_t)y * w * 4, rgba.begin() + (size_t)(y + 1) * w * 4);
    }
    std::vector<uint8_t> z = {0x78, 0x01};
    uint32_t a = 1, b = 0;
    for (uint8_t c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    size_t pos = 0;
    do {
        size_t len = std::min<size_t>(65535, raw.size() - pos);
        bool last = pos + len == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)(len & 0xff));
        z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)(~len & 0xff));
        z.push_back((uint8_t)((~len >> 8) & 0xff));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + len);
        pos += len;
    } while (pos < raw.size());
    put32(z, (b << 16) | a);
    std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    std::vector<uint8_t> ihdr;
    put32(ihdr, (uint32_t)w);
    put32(ihdr, (uint32_t)h);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});
    chunk(png, "IHDR", ihdr);
    chunk(png, "IDAT", z);
    chunk(png, "IEND", {});
    FILE *f = fopen(path, "wb");
    if (!f) return fail(KGK_ERR_IO, std::string("kgk_save_png: cannot open ") + path);
    size_t wr = fwrite(png.data(), 1, png.size(), f);
    int cl = fclose(f);
    if (wr != png.size() || cl != 0) return fail(KGK_ERR_IO, std::string("kgk_save_png: write failed for ") + path);
    return KGK_OK;
    KGK_GUARD_END
}

}  // extern "C"

// OpenEXR output: a single-part scanline file, no compression, channels B, G,
// R (the spec's alphabetical order) as FP32 or FP16, linear values as given.
// No counterpart in the reference (it writes PNG only).
namespace {

// FP32 -> FP16, round to nearest even; overflow to infinity, NaN kept quiet.
uint16_t to_half(float f) {
    uint32_t x;
    memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u | ((ax >> 13) & 0x3ffu) : 0u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);  // rounds to >= 65520: infinity
    if (ax < 0x38800000u) {                                    // below the smallest normal half
        if (ax < 0x33000000u) return (uint16_t)sign;            // below half of the smallest subnormal
        const uint32_t e = ax >> 23, m = (ax & 0x7fffffu) | 0x800000u;
        const uint32_t shift = 126u - e;                        // 14..24
        const uint32_t q = m >> shift, rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1u);
        const uint32_t r = q + (rem > half || (rem == half && (q & 1u)));
        return (uint16_t)(sign | r);
    }
    const uint32_t base = ax - 0x38000000u;  // rebias 127 -> 15
    const uint32_t q = base >> 13, rem = base & 0x1fffu;
    const uint32_t r = q + (rem > 0x1000u || (rem == 0x1000u && (q & 1u)));
    return (uint16_t)(sign | r);
}

void put_le(std::vector<uint8_t> &v, uint64_t x, int bytes) {
    for (int i = 0; i < bytes; ++i) v.push_back((uint8_t)(x >> (8 * i)));
}

void attr(std::vector<uint8_t> &v, const char *name, const char *type, const std::vector<uint8_t> &val) {
    v.insert(v.end(), name, name + strlen(name) + 1);
    v.insert(v.end(), type, type + strlen(type) + 1);
    put_le(v, val.size(), 4);
    v.insert(v.end(), val.begin(), val.end());
}

}  // namespace

extern "C" kgk_status kgk_save_exr(const kgk_vec *img, int32_t w, int32_t h, int32_t half, const char *path) {
    KGK_GUARD_BEGIN
    if (!path || !img) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_save_exr: NULL argument");
    if (w <= 0 || h <= 0) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_save_exr: empty image");
    const size_t n = (size_t)w * h;
    std::vector<kgk_vec> host;
    const kgk_vec *src = img;
    if (is_device_ptr(img)) {
        host.resize(n);
        KGK_CUDA(cudaMemcpy(host.data(), img, n * sizeof(kgk_vec), cudaMemcpyDeviceToHost));
        src = host.data();
    }
    const int ptype = half ? 1 : 2, bpc = half ? 2 : 4;
    std::vector<uint8_t> out = {0x76, 0x2f, 0x31, 0x01, 2, 0, 0, 0};
    std::vector<uint8_t> v;
    for (const char *ch : {"B", "G", "R"}) {
        v.insert(v.end(), ch, ch + 2);
        put_le(v, (uint64_t)ptype, 4);
        v.insert(v.end(), {0, 0, 0, 0});  // pLinear, reserved
        put_le(v, 1, 4);
        put_le(v, 1, 4);
    }
    v.push_back(0);
    attr(out, "channels", "chlist", v);
    attr(out, "compression", "compression", {0});
    v.clear();
    for (int32_t c : {0, 0, w - 1, h - 1}) put_le(v, (uint32_t)c, 4);
    attr(out, "dataWindow", "box2i", v);
    attr(out, "displayWindow", "box2i", v);
    attr(out, "lineOrder", "lineOrder", {0});
    v.clear();
    const float one = 1.0f, zero = 0.0f;
    uint32_t bits;
    memcpy(&bits, &one, 4);
    put_le(v, bits, 4);
    attr(out, "pixelAspectRatio", "float", v);
    v.clear();
    memcpy(&bits, &zero, 4);
    put_le(v, bits, 4);
    put_le(v, bits, 4);
    attr(out, "screenWindowCenter", "v2f", v);
    v.clear();
    memcpy(&bits, &one, 4);
    put_le(v, bits, 4);
    attr(out, "screenWindowWidth", "float", v);
    out.push_back(0);  // end of header
    const size_t line_bytes = (size_t)w * 3 * bpc;
    const size_t table = out.size(), first = table + 8 * (size_t)h;
    for (int y = 0; y < h; ++y) put_le(out, first + (size_t)y * (8 + line_bytes), 8);
    out.reserve(first + (size_t)h * (8 + line_bytes));
    for (int y = 0; y < h; ++y) {
        put_le(out, (uint32_t)y, 4);
        put_le(out, line_bytes, 4);
        const kgk_vec *row = src + (size_t)y * w;
        for (int c = 0; c < 3; ++c) {  // B, G, R
            for (int x = 0; x < w; ++x) {
                const float f = c == 0 ? row[x].z : (c == 1 ? row[x].y : row[x].x);
                if (half) {
                    put_le(out, to_half(f), 2);
                } else {
                    memcpy(&bits, &f, 4);
                    put_le(out, bits, 4);
                }
            }
        }
    }
    FILE *f = fopen(path, "wb");
    if (!f) return fail(KGK_ERR_IO, std::string("kgk_save_exr: cannot open ") + path);
    const size_t wr = fwrite(out.data(), 1, out.size(), f);
    const int cl = fclose(f);
    if (wr != out.size() || cl != 0) return fail(KGK_ERR_IO, std::string("kgk_save_exr: write failed for ") + path);
    return KGK_OK;
    KGK_GUARD_END
}

