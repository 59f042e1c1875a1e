// image_load.cpp - image decoding for scene loading (replaces the stb_image
// calls of FileIO/IO_load_images.cuh:9-19: stbi_loadf with the file's own
// channel count).
//
// The reference loads every texture and the environment with stb_image
// v2.27's stbi_loadf, whose output is:
//   * Radiance .hdr (RGBE, flat or run-length scanlines): 3 float channels,
//     value = byte * 2^(e - 136), 0 when e == 0;
//   * 8-bit images: n_out channels, colour = (byte / 255)^2.2 computed in
//     float, alpha (the last channel when the count is even) = byte / 255;
//   * 16-bit images are first reduced to 8 bits (the high byte).
// This file decodes PNG (every colour type and bit depth, tRNS, Adam7),
// binary PNM (P5 / P6) and Radiance .hdr, takes JPEG from jpeg_load.cpp and
// BMP, GIF, PSD, PIC and TGA from image_formats.cpp, tries the formats in
// stb's order (stbi__load_main: PNG, BMP, GIF, PSD, PIC, JPEG, PNM, then the
// weak TGA test last; .hdr first, as stbi_loadf does) and converts the bytes
// by those rules.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "kgk_scene.h"

using namespace kgk;

namespace {

bool read_file(const char *path, std::vector<uint8_t> &out) {
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    uint8_t buf[1 << 16];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) out.insert(out.end(), buf, buf + n);
    fclose(f);
    return true;
}

// ---------------------------------------------------------------------------
// DEFLATE (RFC 1951) inflater over an in-memory zlib stream (RFC 1950).
// ---------------------------------------------------------------------------
struct BitReader {
    const uint8_t *p;
    size_t n, pos = 0;
    uint32_t bits = 0;
    int count = 0;
    bool over = false;
    int bit() {
        if (count == 0) {
            if (pos >= n) { over = true; return 0; }
            bits = p[pos++];
            count = 8;
        }
        const int b = bits & 1;
        bits >>= 1;
        --count;
        return b;
    }
    uint32_t take(int k) {  // k bits, least significant first
        uint32_t v = 0;
        for (int i = 0; i < k; ++i) v |= (uint32_t)bit() << i;
        return v;
    }
    void align() { count = 0; }
};

// Canonical Huffman decoding table (counts per length + symbols by code).
struct Huffman {
    uint16_t count[16] = {};
    std::vector<uint16_t> symbol;
    bool build(const uint8_t *lengths, int n) {
        symbol.assign(n, 0);
        for (int i = 0; i < 16; ++i) count[i] = 0;
        for (int i = 0; i < n; ++i) ++count[lengths[i]];
        count[0] = 0;
        int left = 1;
        for (int len = 1; len < 16; ++len) {
            left <<= 1;
            left -= count[len];
            if (left < 0) return false;  // over-subscribed
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int len = 1; len < 15; ++len) offs[len + 1] = offs[len] + count[len];
        for (int i = 0; i < n; ++i)
            if (lengths[i]) symbol[offs[lengths[i]]++] = (uint16_t)i;
        return true;
    }
    int decode(BitReader &br) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; ++len) {
            code |= br.bit();
            const int c = count[len];
            if (code - c < first) return symbol[index + (code - first)];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
            if (br.over) return -1;
        }
        return -1;
    }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59,
                               67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769,
                                1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11,
                                12, 12, 13, 13};

bool inflate_block(BitReader &br, const Huffman &lit, const Huffman &dist, std::vector<uint8_t> &out) {
    for (;;) {
        const int sym = lit.decode(br);
        if (sym < 0) return false;
        if (sym < 256) {
            out.push_back((uint8_t)sym);
        } else if (sym == 256) {
            return true;
        } else {
            const int li = sym - 257;
            if (li >= 29) return false;
            const size_t len = kLenBase[li] + br.take(kLenExtra[li]);
            const int ds = dist.decode(br);
            if (ds < 0 || ds >= 30) return false;
            const size_t d = kDistBase[ds] + br.take(kDistExtra[ds]);
            if (d > out.size() || br.over) return false;
            const size_t from = out.size() - d;
            for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);
        }
    }
}

bool zlib_inflate(const std::vector<uint8_t> &in, std::vector<uint8_t> &out, std::string &err) {
    if (in.size() < 2) { err = "zlib stream too short"; return false; }
    const int cmf = in[0], flg = in[1];
    if ((cmf & 15) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 32)) { err = "bad zlib header"; return false; }
    BitReader br{in.data() + 2, in.size() - 2};
    Huffman fixed_lit, fixed_dist;
    {
        uint8_t l[288];
        for (int i = 0; i < 144; ++i) l[i] = 8;
        for (int i = 144; i < 256; ++i) l[i] = 9;
        for (int i = 256; i < 280; ++i) l[i] = 7;
        for (int i = 280; i < 288; ++i) l[i] = 8;
        fixed_lit.build(l, 288);
        uint8_t d[30];
        for (int i = 0; i < 30; ++i) d[i] = 5;
        fixed_dist.build(d, 30);
    }
    int last = 0;
    while (!last) {
        last = (int)br.take(1);
        const int type = (int)br.take(2);
        if (br.over) { err = "truncated deflate stream"; return false; }
        if (type == 0) {
            br.align();
            if (br.pos + 4 > br.n) { err = "truncated stored block"; return false; }
            const size_t len = br.p[br.pos] | (br.p[br.pos + 1] << 8);
            const size_t nlen = br.p[br.pos + 2] | (br.p[br.pos + 3] << 8);
            br.pos += 4;
            if ((len ^ 0xffff) != nlen || br.pos + len > br.n) { err = "bad stored block"; return false; }
            out.insert(out.end(), br.p + br.pos, br.p + br.pos + len);
            br.pos += len;
        } else if (type == 1) {
            if (!inflate_block(br, fixed_lit, fixed_dist, out)) { err = "bad fixed-Huffman block"; return false; }
        } else if (type == 2) {
            const int hlit = (int)br.take(5) + 257, hdist = (int)br.take(5) + 1, hclen = (int)br.take(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {};
            for (int i = 0; i < hclen; ++i) cl[order[i]] = (uint8_t)br.take(3);
            Huffman clh;
            if (!clh.build(cl, 19)) { err = "bad code-length code"; return false; }
            uint8_t lens[320] = {};
            int k = 0;
            while (k < hlit + hdist) {
                const int sym = clh.decode(br);
                if (sym < 0) { err = "bad code lengths"; return false; }
                if (sym < 16) {
                    lens[k++] = (uint8_t)sym;
                } else {
                    int rep = 0;
                    uint8_t val = 0;
                    if (sym == 16) {
                        if (k == 0) { err = "bad code lengths"; return false; }
                        val = lens[k - 1];
                        rep = 3 + (int)br.take(2);
                    } else if (sym == 17) {
                        rep = 3 + (int)br.take(3);
                    } else {
                        rep = 11 + (int)br.take(7);
                    }
                    if (k + rep > hlit + hdist) { err = "bad code lengths"; return false; }
                    while (rep--) lens[k++] = val;
                }
            }
            Huffman lit, dist;
            if (!lit.build(lens, hlit) || !dist.build(lens + hlit, hdist)) { err = "bad Huffman lengths"; return false; }
            if (!inflate_block(br, lit, dist, out)) { err = "bad dynamic-Huffman block"; return false; }
        } else {
            err = "bad deflate block type";
            return false;
        }
    }
    return true;
}

// ---------------------------------------------------------------------------
// PNG
// ---------------------------------------------------------------------------
uint32_t be32(const uint8_t *p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

int paeth(int a, int b, int c) {
    const int p = a + b - c, pa = abs(p - a), pb = abs(p - b), pc = abs(p - c);
    if (pa <= pb && pa <= pc) return a;
    if (pb <= pc) return b;
    return c;
}

// Unfilters one (sub-)image of w x h pixels from `src` (filter byte + row
// bytes per row) into 8-bit samples, 8 bits per channel (16-bit samples keep
// their high byte; 1/2/4-bit grey is scaled to 0..255, palette indices kept).
bool png_unfilter(const uint8_t *&src, const uint8_t *end, uint32_t w, uint32_t h, int channels, int depth,
                  bool scale_low, std::vector<uint16_t> &samples) {
    const size_t bits_pp = (size_t)channels * depth;
    const size_t row_bytes = (w * bits_pp + 7) / 8;
    const size_t bpp = std::max<size_t>(1, bits_pp / 8);
    std::vector<uint8_t> prev(row_bytes, 0), cur(row_bytes);
    samples.assign((size_t)w * h * channels, 0);
    static const int scale_tab[9] = {0, 0xff, 0x55, 0, 0x11, 0, 0, 0, 0x01};
    for (uint32_t y = 0; y < h; ++y) {
        if (src + 1 + row_bytes > end) return false;
        const int ft = *src++;
        for (size_t i = 0; i < row_bytes; ++i) {
            const int x = src[i];
            const int a = i >= bpp ? cur[i - bpp] : 0, b = prev[i], c = i >= bpp ? prev[i - bpp] : 0;
            int v;
            switch (ft) {
                case 0: v = x; break;
                case 1: v = x + a; break;
                case 2: v = x + b; break;
                case 3: v = x + ((a + b) >> 1); break;
                case 4: v = x + paeth(a, b, c); break;
                default: return false;
            }
            cur[i] = (uint8_t)v;
        }
        src += row_bytes;
        uint16_t *out = &samples[(size_t)y * w * channels];
        if (depth == 16) {
            for (size_t i = 0; i < (size_t)w * channels; ++i) out[i] = (uint16_t)(cur[2 * i] << 8 | cur[2 * i + 1]);
        } else if (depth == 8) {
            for (size_t i = 0; i < (size_t)w * channels; ++i) out[i] = cur[i];
        } else {
            const int per = 8 / depth, mask = (1 << depth) - 1;
            const int scale = scale_low ? scale_tab[depth] : 1;
            for (size_t i = 0; i < (size_t)w * channels; ++i) {
                const int byte = cur[i / per], shift = 8 - depth * (int)(i % per + 1);
                out[i] = (uint16_t)(((byte >> shift) & mask) * scale);
            }
        }
        std::swap(prev, cur);
    }
    return true;
}

kgk_status decode_png(const std::vector<uint8_t> &f, int *w_out, int *h_out, int *n_out,
                      std::vector<uint8_t> &pix, const char *path) {
    const std::string where = std::string("png ") + path + ": ";
    size_t pos = 8;
    uint32_t W = 0, H = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, plte, trns;
    bool have_trns = false;
    while (pos + 12 <= f.size()) {
        const uint32_t len = be32(&f[pos]);
        if (pos + 12 + (size_t)len > f.size()) return fail(KGK_ERR_PARSE, where + "truncated chunk");
        const uint8_t *type = &f[pos + 4], *data = &f[pos + 8];
        if (!memcmp(type, "IHDR", 4)) {
            if (len < 13) return fail(KGK_ERR_PARSE, where + "bad IHDR");
            W = be32(data);
            H = be32(data + 4);
            depth = data[8];
            ctype = data[9];
            interlace = data[12];
            if (data[10] != 0 || data[11] != 0 || interlace > 1) return fail(KGK_ERR_PARSE, where + "bad IHDR");
        } else if (!memcmp(type, "PLTE", 4)) {
            plte.assign(data, data + len);
        } else if (!memcmp(type, "tRNS", 4)) {
            trns.assign(data, data + len);
            have_trns = true;
        } else if (!memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), data, data + len);
        } else if (!memcmp(type, "IEND", 4)) {
            break;
        } else if (!memcmp(type, "CgBI", 4)) {
            return fail(KGK_ERR_UNSUPPORTED, where + "Apple CgBI PNG");
        } else if (!(type[0] & 32)) {
            return fail(KGK_ERR_PARSE, where + "unknown critical chunk");
        }
        pos += 12 + len;
    }
    if (W == 0 || H == 0 || W > (1u << 24) || H > (1u << 24)) return fail(KGK_ERR_PARSE, where + "bad size");
    int channels;
    switch (ctype) {
        case 0: channels = 1; break;
        case 2: channels = 3; break;
        case 3: channels = 1; break;
        case 4: channels = 2; break;
        case 6: channels = 4; break;
        default: return fail(KGK_ERR_PARSE, where + "bad colour type");
    }
    const bool depth_ok = depth == 8 || depth == 16 || ((ctype == 0 || ctype == 3) && (depth == 1 || depth == 2 || depth == 4));
    if (!depth_ok || (ctype == 3 && depth == 16)) return fail(KGK_ERR_PARSE, where + "bad bit depth");
    // stb_image's header rule (stbi__parse_png_file): width x height x channels
    // (4 for a paletted image, which expands to RGBA) must stay within 2^30,
    // checked before anything of the image's size is allocated.
    if ((1u << 30) / W / (ctype == 3 ? 4u : (uint32_t)channels) < H) return fail(KGK_ERR_PARSE, where + "too large");
    std::vector<uint8_t> raw;
    std::string zerr;
    if (!zlib_inflate(idat, raw, zerr)) return fail(KGK_ERR_PARSE, where + zerr);
    // decode into samples (full image)
    std::vector<uint16_t> img((size_t)W * H * channels);
    const uint8_t *src = raw.data(), *end = raw.data() + raw.size();
    const bool scale_low = ctype == 0;
    if (!interlace) {
        if (!png_unfilter(src, end, W, H, channels, depth, scale_low, img)) return fail(KGK_ERR_PARSE, where + "bad image data");
    } else {
        static const int xo[7] = {0, 4, 0, 2, 0, 1, 0}, yo[7] = {0, 0, 4, 0, 2, 0, 1};
        static const int xs[7] = {8, 8, 4, 4, 2, 2, 1}, ys[7] = {8, 8, 8, 4, 4, 2, 2};
        for (int p = 0; p < 7; ++p) {
            const uint32_t pw = (W - xo[p] + xs[p] - 1) / xs[p], ph = (H - yo[p] + ys[p] - 1) / ys[p];
            if (W <= (uint32_t)xo[p] || H <= (uint32_t)yo[p] || pw == 0 || ph == 0) continue;
            std::vector<uint16_t> sub;
            if (!png_unfilter(src, end, pw, ph, channels, depth, scale_low, sub)) return fail(KGK_ERR_PARSE, where + "bad image data");
            for (uint32_t j = 0; j < ph; ++j)
                for (uint32_t i = 0; i < pw; ++i)
                    for (int c = 0; c < channels; ++c)
                        img[((size_t)(j * ys[p] + yo[p]) * W + i * xs[p] + xo[p]) * channels + c] =
                            sub[((size_t)j * pw + i) * channels + c];
        }
    }
    const size_t npx = (size_t)W * H;
    int n;
    if (ctype == 3) {
        n = have_trns ? 4 : 3;
        if (plte.size() < 3 || plte.size() % 3) return fail(KGK_ERR_PARSE, where + "bad palette");
        const size_t ne = plte.size() / 3;
        pix.assign(npx * n, 0);
        for (size_t i = 0; i < npx; ++i) {
            const size_t k = img[i];
            if (k >= ne) return fail(KGK_ERR_PARSE, where + "palette index out of range");
            for (int c = 0; c < 3; ++c) pix[i * n + c] = plte[3 * k + c];
            if (n == 4) pix[i * n + 3] = k < trns.size() ? trns[k] : 255;
        }
    } else {
        const bool key = have_trns && (ctype == 0 || ctype == 2);
        n = channels + (key ? 1 : 0);
        pix.assign(npx * n, 0);
        uint16_t kv[3] = {0, 0, 0};
        if (key) {
            static const int scale_tab[9] = {0, 0xff, 0x55, 0, 0x11, 0, 0, 0, 0x01};
            for (int c = 0; c < channels; ++c) {
                if (trns.size() < (size_t)(2 * c + 2)) return fail(KGK_ERR_PARSE, where + "bad tRNS");
                const uint16_t v = (uint16_t)(trns[2 * c] << 8 | trns[2 * c + 1]);
                kv[c] = depth == 16 ? v : (uint16_t)((v & 255) * (depth < 8 ? scale_tab[depth] : 1));
            }
        }
        for (size_t i = 0; i < npx; ++i) {
            bool match = key;
            for (int c = 0; c < channels; ++c) {
                const uint16_t v = img[i * channels + c];
                pix[i * n + c] = (uint8_t)(depth == 16 ? v >> 8 : v);
                if (key && v != kv[c]) match = false;
            }
            if (key) pix[i * n + channels] = match ? 0 : 255;
        }
    }
    *w_out = (int)W;
    *h_out = (int)H;
    *n_out = n;
    return KGK_OK;
}

// ---------------------------------------------------------------------------
// Binary PNM (P5 grey, P6 RGB); samples are taken as stored (no maxval
// scaling), as stb_image does.
// ---------------------------------------------------------------------------
kgk_status decode_pnm(const std::vector<uint8_t> &f, int *w_out, int *h_out, int *n_out, std::vector<uint8_t> &pix,
                      const char *path) {
    const std::string where = std::string("pnm ") + path + ": ";
    size_t pos = 2;
    auto skip = [&]() {
        while (pos < f.size()) {
            if (f[pos] == '#') {
                while (pos < f.size() && f[pos] != '\n' && f[pos] != '\r') ++pos;
            } else if (f[pos] == ' ' || f[pos] == '\t' || f[pos] == '\n' || f[pos] == '\r' || f[pos] == '\v' ||
                       f[pos] == '\f') {
                ++pos;
            } else {
                break;
            }
        }
    };
    auto num = [&](long &v) {
        skip();
        v = 0;
        bool any = false;
        while (pos < f.size() && f[pos] >= '0' && f[pos] <= '9') {
            v = v * 10 + (f[pos++] - '0');
            any = true;
            if (v > (1 << 24)) return false;
        }
        return any;
    };
    const int n = f[1] == '5' ? 1 : 3;
    long w, h, maxv;
    if (!num(w) || !num(h) || !num(maxv) || w <= 0 || h <= 0 || maxv <= 0 || maxv > 65535)
        return fail(KGK_ERR_PARSE, where + "bad header");
    ++pos;  // one whitespace byte
    const int bytes = maxv > 255 ? 2 : 1;
    const size_t cnt = (size_t)w * h * n;
    if (pos + cnt * bytes > f.size()) return fail(KGK_ERR_PARSE, where + "truncated");
    pix.resize(cnt);
    // 16-bit samples: stb_image v2.27 stores the file's big-endian pairs as
    // native (little-endian) 16-bit words and keeps their high byte, i.e. the
    // second byte of each pair
    for (size_t i = 0; i < cnt; ++i) pix[i] = f[pos + i * bytes + (bytes - 1)];
    *w_out = (int)w;
    *h_out = (int)h;
    *n_out = n;
    return KGK_OK;
}

// ---------------------------------------------------------------------------
// Radiance .hdr (RGBE)
// ---------------------------------------------------------------------------
inline void rgbe_to_float(const uint8_t *e, float *out) {
    if (e[3] != 0) {
        const float f1 = (float)ldexp(1.0f, e[3] - (int)(128 + 8));
        out[0] = e[0] * f1;
        out[1] = e[1] * f1;
        out[2] = e[2] * f1;
    } else {
        out[0] = out[1] = out[2] = 0.0f;
    }
}

kgk_status decode_hdr(const std::vector<uint8_t> &f, kgk_texture *out, const char *path) {
    const std::string where = std::string("hdr ") + path + ": ";
    size_t pos = 0;
    auto line = [&]() {
        std::string s;
        while (pos < f.size() && f[pos] != '\n') s += (char)f[pos++];
        if (pos < f.size()) ++pos;
        return s;
    };
    const std::string id = line();
    if (id != "#?RADIANCE" && id != "#?RGBE") return fail(KGK_ERR_PARSE, where + "not a Radiance file");
    bool valid = false;
    for (;;) {
        const std::string t = line();
        if (t.empty()) break;
        if (t == "FORMAT=32-bit_rle_rgbe") valid = true;
    }
    if (!valid) return fail(KGK_ERR_UNSUPPORTED, where + "only FORMAT=32-bit_rle_rgbe is supported");
    const std::string dims = line();
    if (dims.compare(0, 3, "-Y ") != 0) return fail(KGK_ERR_UNSUPPORTED, where + "unsupported data layout");
    char *p = const_cast<char *>(dims.c_str()) + 3;
    const long H = strtol(p, &p, 10);
    while (*p == ' ') ++p;
    if (strncmp(p, "+X ", 3) != 0) return fail(KGK_ERR_UNSUPPORTED, where + "unsupported data layout");
    const long W = strtol(p + 3, nullptr, 10);
    if (W <= 0 || H <= 0 || W > (1 << 24) || H > (1 << 24)) return fail(KGK_ERR_PARSE, where + "bad size");
    // stb_image's stbi__mad4sizes_valid: width x height x 3 floats must fit in an int.
    if ((uint64_t)W * (uint64_t)H * 3u * sizeof(float) > 0x7fffffffull) return fail(KGK_ERR_PARSE, where + "too large");
    float *px = (float *)malloc((size_t)W * H * 3 * sizeof(float));
    if (!px) return fail(KGK_ERR_OUT_OF_MEMORY, where + "out of host memory");
    auto bad = [&](const char *m) {
        free(px);
        return fail(KGK_ERR_PARSE, where + m);
    };
    auto get = [&](uint8_t *b, size_t k) {
        if (pos + k > f.size()) return false;
        memcpy(b, &f[pos], k);
        pos += k;
        return true;
    };
    // Flat pixels from pixel index `from` to the end.
    auto flat = [&](size_t from) {
        for (size_t i = from; i < (size_t)W * H; ++i) {
            uint8_t e[4];
            if (!get(e, 4)) return false;
            rgbe_to_float(e, px + 3 * i);
        }
        return true;
    };
    if (W < 8 || W >= 32768) {
        if (!flat(0)) return bad("truncated pixel data");
    } else {
        std::vector<uint8_t> scan((size_t)W * 4);
        for (long j = 0; j < H; ++j) {
            uint8_t hd[4];
            if (!get(hd, 3)) return bad("truncated pixel data");
            if (hd[0] != 2 || hd[1] != 2 || (hd[2] & 0x80)) {
                // not run-length encoded: the file is flat from here, these
                // bytes being the first pixel (read as pixel 0 of the image)
                if (!get(hd + 3, 1)) return bad("truncated pixel data");
                rgbe_to_float(hd, px);
                if (!flat(1)) return bad("truncated pixel data");
                break;
            }
            uint8_t lo;
            if (!get(&lo, 1)) return bad("truncated pixel data");
            if (((long)hd[2] << 8 | lo) != W) return bad("bad scanline length");
            for (int k = 0; k < 4; ++k) {
                long i = 0;
                while (W - i > 0) {
                    uint8_t cnt;
                    if (!get(&cnt, 1)) return bad("truncated pixel data");
                    if (cnt > 128) {
                        uint8_t v;
                        if (!get(&v, 1)) return bad("truncated pixel data");
                        cnt -= 128;
                        if (cnt > W - i) return bad("bad run length");
                        for (int z = 0; z < cnt; ++z) scan[(i++) * 4 + k] = v;
                    } else {
                        if (cnt > W - i) return bad("bad run length");
                        for (int z = 0; z < cnt; ++z) {
                            if (!get(&scan[(i++) * 4 + k], 1)) return bad("truncated pixel data");
                        }
                    }
                }
            }
            for (long i = 0; i < W; ++i) rgbe_to_float(&scan[i * 4], px + 3 * ((size_t)j * W + i));
        }
    }
    out->pixels = px;
    out->width = (int32_t)W;
    out->height = (int32_t)H;
    out->bpp = 3;
    return KGK_OK;
}

// A JPEG starts with 0xff (more 0xff fill bytes may follow) and the SOI marker.
bool is_jpeg(const std::vector<uint8_t> &f) {
    if (f.empty() || f[0] != 0xff) return false;
    size_t i = 1;
    while (i < f.size() && f[i] == 0xff) ++i;
    return i < f.size() && f[i] == 0xd8;
}

}  // namespace

namespace kgk {

kgk_status decode_jpeg(const std::vector<uint8_t> &f, int *w_out, int *h_out, int *n_out, std::vector<uint8_t> &pix,
                       const char *path);
// image_formats.cpp
bool is_bmp(const std::vector<uint8_t> &f);
bool is_gif(const std::vector<uint8_t> &f);
bool is_psd(const std::vector<uint8_t> &f);
bool is_pic(const std::vector<uint8_t> &f);
bool is_tga(const std::vector<uint8_t> &f);
kgk_status decode_bmp(const std::vector<uint8_t> &f, int *w, int *h, int *n, std::vector<uint8_t> &pix, const char *path);
kgk_status decode_gif(const std::vector<uint8_t> &f, int *w, int *h, int *n, std::vector<uint8_t> &pix, const char *path);
kgk_status decode_psd(const std::vector<uint8_t> &f, int *w, int *h, int *n, std::vector<uint8_t> &pix, const char *path);
kgk_status decode_pic(const std::vector<uint8_t> &f, int *w, int *h, int *n, std::vector<uint8_t> &pix, const char *path);
kgk_status decode_tga(const std::vector<uint8_t> &f, int *w, int *h, int *n, std::vector<uint8_t> &pix, const char *path);

// stbi_loadf: decode and convert to float (see the file comment).
kgk_status load_image_float(const char *path, kgk_texture *out) {
    out->pixels = nullptr;
    out->width = out->height = out->bpp = 0;
    std::vector<uint8_t> f;
    if (!read_file(path, f)) return fail(KGK_ERR_IO, std::string("cannot open image ") + path);
    static const char *kHdr1 = "#?RADIANCE\n", *kHdr2 = "#?RGBE\n";
    if ((f.size() >= 11 && !memcmp(f.data(), kHdr1, 11)) || (f.size() >= 7 && !memcmp(f.data(), kHdr2, 7)))
        return decode_hdr(f, out, path);
    int w = 0, h = 0, n = 0;
    std::vector<uint8_t> pix;
    static const uint8_t kPng[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (f.size() >= 8 && !memcmp(f.data(), kPng, 8)) {
        KGK_TRY(decode_png(f, &w, &h, &n, pix, path));
    } else if (is_bmp(f)) {
        KGK_TRY(decode_bmp(f, &w, &h, &n, pix, path));
    } else if (is_gif(f)) {
        KGK_TRY(decode_gif(f, &w, &h, &n, pix, path));
    } else if (is_psd(f)) {
        KGK_TRY(decode_psd(f, &w, &h, &n, pix, path));
    } else if (is_pic(f)) {
        KGK_TRY(decode_pic(f, &w, &h, &n, pix, path));
    } else if (is_jpeg(f)) {
        KGK_TRY(decode_jpeg(f, &w, &h, &n, pix, path));
    } else if (f.size() >= 3 && f[0] == 'P' && (f[1] == '5' || f[1] == '6')) {
        KGK_TRY(decode_pnm(f, &w, &h, &n, pix, path));
    } else if (is_tga(f)) {
        KGK_TRY(decode_tga(f, &w, &h, &n, pix, path));
    } else {
        return fail(KGK_ERR_UNSUPPORTED, std::string("unknown image format: ") + path);
    }
    const size_t npx = (size_t)w * h;
    float *px = (float *)malloc(npx * n * sizeof(float));
    if (!px) return fail(KGK_ERR_OUT_OF_MEMORY, "image: out of host memory");
    const int nc = (n & 1) ? n : n - 1;  // colour channels; the last is alpha when n is even
    for (size_t i = 0; i < npx; ++i) {
        for (int k = 0; k < nc; ++k) px[i * n + k] = (float)powf(pix[i * n + k] / 255.0f, 2.2f);
        if (nc < n) px[i * n + nc] = pix[i * n + nc] / 255.0f;
    }
    out->pixels = px;
    out->width = w;
    out->height = h;
    out->bpp = n;
    return KGK_OK;
}

}  // namespace kgk

extern "C" {

kgk_status kgk_load_image(const char *path, kgk_texture *out) {
    KGK_GUARD_BEGIN
    if (!path || !out) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_load_image: NULL argument");
    return load_image_float(path, out);
    KGK_GUARD_END
}

void kgk_image_free(kgk_texture *t) {
    if (!t) return;
    free(t->pixels);
    t->pixels = nullptr;
    t->width = t->height = t->bpp = 0;
}

}  // extern "C"
