// image_formats.cpp - the remaining 8-bit formats that stb_image v2.27's
// stbi_loadf accepts for textures (FileIO/IO_load_images.cuh:9-19): BMP, TGA,
// GIF (first frame), PSD and Softimage PIC.  Each decoder restates the
// behaviour of the vendored stb_image.h (external_lib/stb/stb_image.h, the
// line ranges cited per function) so that the bytes handed to the float
// conversion in image_load.cpp are the same, including its quirks:
//   * reads past the end of the file yield 0 (stb's buffered file reader);
//   * BMP: the OS/2 (12-byte header) palette size formula, the all-zero alpha
//     rule, bottom-up rows flipped;
//   * GIF: pixels not drawn by the first frame take the background palette
//     entry in its stored (B, G, R) order, alpha 255;
//   * PSD: always four channels, the "white matte" removal in FP32.
// Output: w x h x n bytes, n as stb reports it (the float conversion keeps
// that channel count).
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "kgk_scene.h"

namespace kgk {
namespace {

constexpr uint32_t kMaxDim = 1u << 24;  // stb's STBI_MAX_DIMENSIONS

// stb's stbi__mad3sizes_valid: w * h * n bytes must fit in an int.
bool too_large(uint64_t w, uint64_t h, uint64_t n) { return w * h * n > 0x7fffffffull; }

// Sequential reader with stb's end-of-file behaviour.
struct Rd {
    const uint8_t *p;
    size_t n, pos = 0;
    Rd(const std::vector<uint8_t> &f) : p(f.data()), n(f.size()) {}
    int get8() {
        const int v = pos < n ? p[pos] : 0;
        ++pos;
        return v;
    }
    uint32_t le16() {
        const uint32_t a = (uint32_t)get8();
        return a | (uint32_t)get8() << 8;
    }
    uint32_t le32() {
        const uint32_t a = le16();
        return a | le16() << 16;
    }
    uint32_t be16() {
        const uint32_t a = (uint32_t)get8();
        return a << 8 | (uint32_t)get8();
    }
    uint32_t be32() {
        const uint32_t a = be16();
        return a << 16 | be16();
    }
    // stbi__skip: a negative count moves to the end
    void skip(long long k) {
        if (k < 0) pos = n > pos ? n : pos;
        else pos += (size_t)k;
    }
    bool eof() const { return pos >= n; }
    // stbi__getn: true when all k bytes were there; copies what there is
    bool getn(uint8_t *dst, size_t k) {
        const size_t have = pos < n ? std::min(k, n - pos) : 0;
        if (have) memcpy(dst, p + pos, have);
        pos += k;
        return have == k;
    }
};

// ---------------------------------------------------------------------------
// BMP (stb_image.h:5282-5655)
// ---------------------------------------------------------------------------
int high_bit(uint32_t z) {
    if (z == 0) return -1;
    int n = 0;
    while (z >>= 1) ++n;
    return n;
}

int bit_count(uint32_t a) {
    int c = 0;
    for (; a; a &= a - 1) ++c;
    return c;
}

// The masked field moved so its top bit is bit 7, cut to `bits` bits and
// widened to 8 by bit replication (stbi__shiftsigned, stb_image.h:5328-5347).
int shift_signed(uint32_t v, int shift, int bits) {
    static const unsigned mul[9] = {0, 0xff, 0x55, 0x49, 0x11, 0x21, 0x41, 0x81, 0x01};
    static const unsigned sh[9] = {0, 0, 0, 1, 0, 2, 4, 6, 0};
    if (shift < 0) v <<= -shift;
    else v >>= shift;
    v >>= (8 - bits);
    return (int)((v & 0xffu) * mul[bits]) >> sh[bits];
}

}  // namespace

bool is_bmp(const std::vector<uint8_t> &f) {
    Rd r(f);
    if (r.get8() != 'B' || r.get8() != 'M') return false;
    r.skip(12);
    const uint32_t sz = r.le32();
    return sz == 12 || sz == 40 || sz == 56 || sz == 108 || sz == 124;
}

kgk_status decode_bmp(const std::vector<uint8_t> &f, int *w_out, int *h_out, int *n_out, std::vector<uint8_t> &pix,
                      const char *path) {
    const std::string where = std::string("bmp ") + path + ": ";
    Rd r(f);
    r.skip(2 + 4 + 4);
    const int32_t offset = (int32_t)r.le32();
    const uint32_t hsz = r.le32();
    uint32_t mr = 0, mg = 0, mb = 0, ma = 0, all_a = 255;
    int extra_read = 14;
    if (offset < 0) return fail(KGK_ERR_PARSE, where + "bad data offset");
    uint32_t w, hraw;
    if (hsz == 12) {
        w = r.le16();
        hraw = r.le16();
    } else {
        w = r.le32();
        hraw = r.le32();
    }
    if (r.le16() != 1) return fail(KGK_ERR_PARSE, where + "planes != 1");
    const int bpp = (int)r.le16();
    auto defaults = [&](uint32_t compress) {
        if (compress == 3) return;
        if (bpp == 16) {
            mr = 31u << 10;
            mg = 31u << 5;
            mb = 31u;
        } else if (bpp == 32) {
            mr = 0xffu << 16;
            mg = 0xffu << 8;
            mb = 0xffu;
            ma = 0xffu << 24;
            all_a = 0;  // loaded alpha that is zero everywhere becomes 255
        } else {
            mr = mg = mb = ma = 0;
        }
    };
    if (hsz != 12) {
        const uint32_t compress = r.le32();
        if (compress == 1 || compress == 2) return fail(KGK_ERR_UNSUPPORTED, where + "RLE compression");
        if (compress >= 4) return fail(KGK_ERR_UNSUPPORTED, where + "JPEG/PNG compression");
        if (compress == 3 && bpp != 16 && bpp != 32) return fail(KGK_ERR_PARSE, where + "bit fields need 16 or 32 bpp");
        r.skip(20);
        if (hsz == 40 || hsz == 56) {
            if (hsz == 56) r.skip(16);
            if (bpp == 16 || bpp == 32) {
                if (compress == 0) {
                    defaults(0);
                } else {  // 3
                    mr = r.le32();
                    mg = r.le32();
                    mb = r.le32();
                    extra_read += 12;
                    if (mr == mg && mg == mb) return fail(KGK_ERR_PARSE, where + "equal bit fields");
                }
            }
        } else if (hsz == 108 || hsz == 124) {
            mr = r.le32();
            mg = r.le32();
            mb = r.le32();
            ma = r.le32();
            if (compress != 3) defaults(compress);
            r.skip(4 + 48);
            if (hsz == 124) r.skip(16);
        } else {
            return fail(KGK_ERR_PARSE, where + "unknown header size");
        }
    }
    const bool flip = (int32_t)hraw > 0;
    const uint32_t h = (uint32_t)std::abs((int32_t)hraw);
    if (h > kMaxDim || w > kMaxDim || w == 0 || h == 0) return fail(KGK_ERR_PARSE, where + "bad dimensions");
    int psize = 0;
    if (hsz == 12) {
        if (bpp < 24) psize = (offset - extra_read - 24) / 3;
    } else if (bpp < 16) {
        psize = (offset - extra_read - (int)hsz) >> 2;
    }
    if (psize == 0 && (size_t)offset != r.pos) return fail(KGK_ERR_PARSE, where + "bad data offset");
    const int img_n = (bpp == 24 && ma == 0xff000000u) ? 3 : (ma ? 4 : 3);
    const int target = img_n;
    if (too_large(w, h, target)) return fail(KGK_ERR_PARSE, where + "too large");
    pix.assign((size_t)w * h * target, 0);
    uint8_t *out = pix.data();
    size_t z = 0;
    if (bpp < 16) {
        if (psize <= 0 || psize > 256) return fail(KGK_ERR_PARSE, where + "bad palette");
        uint8_t pal[256][4] = {};
        for (int i = 0; i < psize; ++i) {
            pal[i][2] = (uint8_t)r.get8();
            pal[i][1] = (uint8_t)r.get8();
            pal[i][0] = (uint8_t)r.get8();
            if (hsz != 12) r.get8();
            pal[i][3] = 255;
        }
        r.skip((long long)offset - extra_read - (long long)hsz - (long long)psize * (hsz == 12 ? 3 : 4));
        int width;
        if (bpp == 1) width = (int)((w + 7) >> 3);
        else if (bpp == 4) width = (int)((w + 1) >> 1);
        else if (bpp == 8) width = (int)w;
        else return fail(KGK_ERR_UNSUPPORTED, where + "bits per pixel");
        const int pad = (-width) & 3;
        auto put = [&](int c) {
            out[z++] = pal[c][0];
            out[z++] = pal[c][1];
            out[z++] = pal[c][2];
            if (target == 4) out[z++] = 255;
        };
        for (uint32_t j = 0; j < h; ++j) {
            if (bpp == 1) {
                int bit = 7, v = r.get8();
                for (uint32_t i = 0; i < w; ++i) {
                    put((v >> bit) & 1);
                    if (i + 1 == w) break;
                    if (--bit < 0) {
                        bit = 7;
                        v = r.get8();
                    }
                }
            } else {
                for (uint32_t i = 0; i < w; i += 2) {
                    int v = r.get8(), v2 = 0;
                    if (bpp == 4) {
                        v2 = v & 15;
                        v >>= 4;
                    }
                    put(v);
                    if (i + 1 == w) break;
                    put(bpp == 8 ? r.get8() : v2);
                }
            }
            r.skip(pad);
        }
    } else {
        r.skip((long long)offset - extra_read - (long long)hsz);
        const int width = bpp == 24 ? 3 * (int)w : bpp == 16 ? 2 * (int)w : 0;
        const int pad = (-width) & 3;
        int easy = 0;
        if (bpp == 24) easy = 1;
        else if (bpp == 32 && mb == 0xff && mg == 0xff00 && mr == 0xff0000 && ma == 0xff000000u) easy = 2;
        int rs = 0, gs = 0, bs = 0, as = 0, rc = 0, gc = 0, bc = 0, ac = 0;
        if (!easy) {
            if (!mr || !mg || !mb) return fail(KGK_ERR_PARSE, where + "bad bit fields");
            rs = high_bit(mr) - 7;
            rc = bit_count(mr);
            gs = high_bit(mg) - 7;
            gc = bit_count(mg);
            bs = high_bit(mb) - 7;
            bc = bit_count(mb);
            as = high_bit(ma) - 7;
            ac = bit_count(ma);
            if (rc > 8 || gc > 8 || bc > 8 || ac > 8) return fail(KGK_ERR_UNSUPPORTED, where + "fields over 8 bits");
        }
        for (uint32_t j = 0; j < h; ++j) {
            for (uint32_t i = 0; i < w; ++i) {
                uint32_t a;
                if (easy) {
                    out[z + 2] = (uint8_t)r.get8();
                    out[z + 1] = (uint8_t)r.get8();
                    out[z + 0] = (uint8_t)r.get8();
                    z += 3;
                    a = easy == 2 ? (uint32_t)r.get8() : 255u;
                } else {
                    const uint32_t v = bpp == 16 ? r.le16() : r.le32();
                    out[z++] = (uint8_t)shift_signed(v & mr, rs, rc);
                    out[z++] = (uint8_t)shift_signed(v & mg, gs, gc);
                    out[z++] = (uint8_t)shift_signed(v & mb, bs, bc);
                    a = ma ? (uint32_t)shift_signed(v & ma, as, ac) : 255u;
                }
                all_a |= a;
                if (target == 4) out[z++] = (uint8_t)a;
            }
            r.skip(pad);
        }
    }
    if (target == 4 && all_a == 0)
        for (size_t i = 3; i < pix.size(); i += 4) out[i] = 255;
    if (flip) {
        const size_t row = (size_t)w * target;
        std::vector<uint8_t> tmp(row);
        for (uint32_t j = 0; j < h / 2; ++j) {
            uint8_t *a = out + j * row, *b = out + (h - 1 - j) * row;
            memcpy(tmp.data(), a, row);
            memcpy(a, b, row);
            memcpy(b, tmp.data(), row);
        }
    }
    *w_out = (int)w;
    *h_out = (int)h;
    *n_out = img_n;
    return KGK_OK;
}

// ---------------------------------------------------------------------------
// GIF, first frame (stb_image.h:6502-6807, 6970-6996)
// ---------------------------------------------------------------------------
bool is_gif(const std::vector<uint8_t> &f) {
    return f.size() >= 6 && !memcmp(f.data(), "GIF8", 4) && (f[4] == '7' || f[4] == '9') && f[5] == 'a';
}

kgk_status decode_gif(const std::vector<uint8_t> &f, int *w_out, int *h_out, int *n_out, std::vector<uint8_t> &pix,
                      const char *path) {
    const std::string where = std::string("gif ") + path + ": ";
    Rd r(f);
    r.skip(6);
    const int W = (int)r.le16(), H = (int)r.le16();
    const int flags = r.get8(), bgindex = r.get8();
    r.get8();  // aspect ratio
    int transparent = -1, eflags = 0;
    if ((uint32_t)W > kMaxDim || (uint32_t)H > kMaxDim || W == 0 || H == 0)
        return fail(KGK_ERR_PARSE, where + "bad dimensions");
    // palettes stored as (B, G, R, A), as stb keeps them
    uint8_t pal[256][4] = {}, lpal[256][4] = {};
    auto colortable = [&](uint8_t (*p)[4], int num, int transp) {
        for (int i = 0; i < num; ++i) {
            p[i][2] = (uint8_t)r.get8();
            p[i][1] = (uint8_t)r.get8();
            p[i][0] = (uint8_t)r.get8();
            p[i][3] = transp == i ? 0 : 255;
        }
    };
    if (too_large((uint32_t)W, (uint32_t)H, 4)) return fail(KGK_ERR_PARSE, where + "too large");
    if (flags & 0x80) colortable(pal, 2 << (flags & 7), -1);
    const size_t pcount = (size_t)W * H;
    pix.assign(pcount * 4, 0);
    std::vector<uint8_t> history(pcount, 0);
    for (;;) {
        const int tag = r.get8();
        if (tag == 0x2C) {
            const int x = (int)r.le16(), y = (int)r.le16(), w = (int)r.le16(), h = (int)r.le16();
            if (x + w > W || y + h > H) return fail(KGK_ERR_PARSE, where + "bad image descriptor");
            const int line = W * 4;
            const int start_x = x * 4, start_y = y * line;
            const int max_x = start_x + w * 4, max_y = start_y + h * line;
            int cur_x = start_x, cur_y = w == 0 ? max_y : start_y;
            const int lflags = r.get8();
            int step, parse;
            if (lflags & 0x40) {
                step = 8 * line;
                parse = 3;
            } else {
                step = line;
                parse = 0;
            }
            const uint8_t (*ct)[4];
            if (lflags & 0x80) {
                colortable(lpal, 2 << (lflags & 7), (eflags & 1) ? transparent : -1);
                ct = lpal;
            } else if (flags & 0x80) {
                ct = pal;
            } else {
                return fail(KGK_ERR_PARSE, where + "missing colour table");
            }
            // LZW raster (stbi__process_gif_raster, stb_image.h:6616-6696)
            const int lzw_cs = r.get8();
            if (lzw_cs > 12) return fail(KGK_ERR_PARSE, where + "bad LZW code size");
            struct Code {
                int16_t prefix;
                uint8_t first, suffix;
            };
            std::vector<Code> codes(8192);
            const int clear = 1 << lzw_cs;
            for (int i = 0; i < clear; ++i) codes[i] = {-1, (uint8_t)i, (uint8_t)i};
            int codesize = lzw_cs + 1, codemask = (1 << codesize) - 1, avail = clear + 2, oldcode = -1;
            bool first = true;
            int32_t bits = 0;
            int valid = 0, len = 0;
            std::vector<uint8_t> chain;
            chain.reserve(8192);
            auto emit = [&](int code) {
                chain.clear();
                for (int c = code; c >= 0; c = codes[c].prefix) chain.push_back(codes[c].suffix);
                for (size_t k = chain.size(); k-- > 0;) {
                    if (cur_y >= max_y) continue;
                    const int idx = cur_x + cur_y;
                    history[idx / 4] = 1;
                    const uint8_t *c = ct[chain[k]];
                    if (c[3] > 128) {
                        pix[idx + 0] = c[2];
                        pix[idx + 1] = c[1];
                        pix[idx + 2] = c[0];
                        pix[idx + 3] = c[3];
                    }
                    cur_x += 4;
                    if (cur_x >= max_x) {
                        cur_x = start_x;
                        cur_y += step;
                        while (cur_y >= max_y && parse > 0) {
                            step = (1 << parse) * line;
                            cur_y = start_y + (step >> 1);
                            --parse;
                        }
                    }
                }
            };
            for (;;) {
                if (valid < codesize) {
                    if (len == 0) {
                        len = r.get8();
                        if (len == 0) break;
                    }
                    --len;
                    bits |= (int32_t)r.get8() << valid;
                    valid += 8;
                    continue;
                }
                const int code = bits & codemask;
                bits >>= codesize;
                valid -= codesize;
                if (code == clear) {
                    codesize = lzw_cs + 1;
                    codemask = (1 << codesize) - 1;
                    avail = clear + 2;
                    oldcode = -1;
                    first = false;
                } else if (code == clear + 1) {
                    r.skip(len);
                    while ((len = r.get8()) > 0) r.skip(len);
                    break;
                } else if (code <= avail) {
                    if (first) return fail(KGK_ERR_PARSE, where + "no clear code");
                    if (oldcode >= 0) {
                        Code &p = codes[avail++];
                        if (avail > 8192) return fail(KGK_ERR_PARSE, where + "too many codes");
                        p.prefix = (int16_t)oldcode;
                        p.first = codes[oldcode].first;
                        p.suffix = code == avail ? p.first : codes[code].first;
                    } else if (code == avail) {
                        return fail(KGK_ERR_PARSE, where + "illegal code");
                    }
                    emit(code);
                    if ((avail & codemask) == 0 && avail <= 0x0fff) {
                        ++codesize;
                        codemask = (1 << codesize) - 1;
                    }
                    oldcode = code;
                } else {
                    return fail(KGK_ERR_PARSE, where + "illegal code");
                }
            }
            // first frame: pixels not drawn take the background entry as stored
            if (bgindex > 0) {
                pal[bgindex][3] = 255;
                for (size_t i = 0; i < pcount; ++i)
                    if (!history[i]) memcpy(&pix[i * 4], pal[bgindex], 4);
            }
            *w_out = W;
            *h_out = H;
            *n_out = 4;
            return KGK_OK;
        } else if (tag == 0x21) {
            const int ext = r.get8();
            if (ext == 0xF9) {
                const int len = r.get8();
                if (len == 4) {
                    eflags = r.get8();
                    r.le16();  // delay
                    if (transparent >= 0) pal[transparent][3] = 255;
                    if (eflags & 1) {
                        transparent = r.get8();
                        pal[transparent][3] = 0;
                    } else {
                        r.skip(1);
                        transparent = -1;
                    }
                } else {
                    r.skip(len);
                    continue;
                }
            }
            int len;
            while ((len = r.get8()) != 0) r.skip(len);
        } else if (tag == 0x3B) {
            return fail(KGK_ERR_PARSE, where + "no image in the file");
        } else {
            return fail(KGK_ERR_PARSE, where + "unknown block");
        }
    }
}

// ---------------------------------------------------------------------------
// PSD (stb_image.h:6003-6246): RGB mode, 8 or 16 bits, raw or RLE; always
// four output channels
// ---------------------------------------------------------------------------
bool is_psd(const std::vector<uint8_t> &f) { return f.size() >= 4 && !memcmp(f.data(), "8BPS", 4); }

kgk_status decode_psd(const std::vector<uint8_t> &f, int *w_out, int *h_out, int *n_out, std::vector<uint8_t> &pix,
                      const char *path) {
    const std::string where = std::string("psd ") + path + ": ";
    Rd r(f);
    r.skip(4);
    if (r.be16() != 1) return fail(KGK_ERR_UNSUPPORTED, where + "version");
    r.skip(6);
    const int channels = (int)r.be16();
    if (channels > 16) return fail(KGK_ERR_UNSUPPORTED, where + "channel count");
    const uint32_t h = r.be32(), w = r.be32();
    if (h > kMaxDim || w > kMaxDim) return fail(KGK_ERR_PARSE, where + "bad dimensions");
    const uint32_t depth = r.be16();
    if (depth != 8 && depth != 16) return fail(KGK_ERR_UNSUPPORTED, where + "bit depth");
    if (r.be16() != 3) return fail(KGK_ERR_UNSUPPORTED, where + "not RGB colour mode");
    for (int k = 0; k < 3; ++k) r.skip((long long)(int32_t)r.be32());  // mode data, resources, reserved
    const uint32_t compression = r.be16();
    if (compression > 1) return fail(KGK_ERR_UNSUPPORTED, where + "compression");
    if (too_large(w, h, 4)) return fail(KGK_ERR_PARSE, where + "too large");
    const size_t count = (size_t)w * h;
    pix.assign(count * 4, 0);
    if (compression) {
        r.skip((long long)h * channels * 2);  // per-row byte counts
        for (int c = 0; c < 4; ++c) {
            uint8_t *p = pix.data() + c;
            if (c >= channels) {
                for (size_t i = 0; i < count; ++i, p += 4) *p = c == 3 ? 255 : 0;
                continue;
            }
            size_t done = 0;
            while (done < count) {
                const size_t left = count - done;
                int len = r.get8();
                if (len == 128) continue;
                if (len < 128) {
                    const size_t n = (size_t)len + 1;
                    if (n > left) return fail(KGK_ERR_PARSE, where + "bad RLE data");
                    for (size_t k = 0; k < n; ++k, p += 4) *p = (uint8_t)r.get8();
                    done += n;
                } else {
                    const size_t n = 257 - (size_t)len;
                    if (n > left) return fail(KGK_ERR_PARSE, where + "bad RLE data");
                    const uint8_t v = (uint8_t)r.get8();
                    for (size_t k = 0; k < n; ++k, p += 4) *p = v;
                    done += n;
                }
            }
        }
    } else {
        for (int c = 0; c < 4; ++c) {
            uint8_t *p = pix.data() + c;
            if (c >= channels) {
                for (size_t i = 0; i < count; ++i, p += 4) *p = c == 3 ? 255 : 0;
            } else if (depth == 16) {
                for (size_t i = 0; i < count; ++i, p += 4) *p = (uint8_t)(r.be16() >> 8);
            } else {
                for (size_t i = 0; i < count; ++i, p += 4) *p = (uint8_t)r.get8();
            }
        }
    }
    if (channels >= 4) {
        // remove the white matte: c' = c / a + 255 (1 - 1 / a), in FP32, truncated
        for (size_t i = 0; i < count; ++i) {
            uint8_t *px = &pix[i * 4];
            if (px[3] != 0 && px[3] != 255) {
                const float a = px[3] / 255.0f;
                const float ra = 1.0f / a;
                const float inv_a = 255.0f * (1 - ra);
                for (int k = 0; k < 3; ++k) px[k] = (uint8_t)(int)((float)px[k] * ra + inv_a);
            }
        }
    }
    *w_out = (int)w;
    *h_out = (int)h;
    *n_out = 4;
    return KGK_OK;
}

// ---------------------------------------------------------------------------
// Softimage PIC (stb_image.h:6258-6464)
// ---------------------------------------------------------------------------
bool is_pic(const std::vector<uint8_t> &f) {
    static const uint8_t magic[4] = {0x53, 0x80, 0xF6, 0x34};
    return f.size() >= 92 && !memcmp(f.data(), magic, 4) && !memcmp(f.data() + 88, "PICT", 4);
}

kgk_status decode_pic(const std::vector<uint8_t> &f, int *w_out, int *h_out, int *n_out, std::vector<uint8_t> &pix,
                      const char *path) {
    const std::string where = std::string("pic ") + path + ": ";
    Rd r(f);
    r.skip(92);
    const uint32_t w = r.be16(), h = r.be16();
    if (r.eof()) return fail(KGK_ERR_PARSE, where + "file too short");
    if (too_large(w, h, 4)) return fail(KGK_ERR_PARSE, where + "too large");
    r.skip(8);  // ratio, fields, pad
    struct Packet {
        int size, type, channel;
    };
    Packet packets[10];
    int npk = 0, act = 0, chained;
    do {
        if (npk == 10) return fail(KGK_ERR_PARSE, where + "too many packets");
        Packet &pk = packets[npk++];
        chained = r.get8();
        pk.size = r.get8();
        pk.type = r.get8();
        pk.channel = r.get8();
        act |= pk.channel;
        if (r.eof()) return fail(KGK_ERR_PARSE, where + "file too short");
        if (pk.size != 8) return fail(KGK_ERR_UNSUPPORTED, where + "packet is not 8 bits per channel");
    } while (chained);
    const int comp = (act & 0x10) ? 4 : 3;
    std::vector<uint8_t> rgba((size_t)w * h * 4, 0xff);
    auto readval = [&](int channel, uint8_t *dest) {
        for (int i = 0, mask = 0x80; i < 4; ++i, mask >>= 1)
            if (channel & mask) {
                if (r.eof()) return false;
                dest[i] = (uint8_t)r.get8();
            }
        return true;
    };
    auto copyval = [](int channel, uint8_t *dest, const uint8_t *src) {
        for (int i = 0, mask = 0x80; i < 4; ++i, mask >>= 1)
            if (channel & mask) dest[i] = src[i];
    };
    for (uint32_t y = 0; y < h; ++y) {
        for (int k = 0; k < npk; ++k) {
            const Packet &pk = packets[k];
            uint8_t *dest = rgba.data() + (size_t)y * w * 4;
            if (pk.type == 0) {
                for (uint32_t x = 0; x < w; ++x, dest += 4)
                    if (!readval(pk.channel, dest)) return fail(KGK_ERR_PARSE, where + "file too short");
            } else if (pk.type == 1) {
                int left = (int)w;
                while (left > 0) {
                    int count = r.get8();
                    if (r.eof()) return fail(KGK_ERR_PARSE, where + "file too short");
                    if (count > left) count = left;
                    uint8_t v[4];
                    if (!readval(pk.channel, v)) return fail(KGK_ERR_PARSE, where + "file too short");
                    for (int i = 0; i < count; ++i, dest += 4) copyval(pk.channel, dest, v);
                    left -= count;
                }
            } else if (pk.type == 2) {
                int left = (int)w;
                while (left > 0) {
                    int count = r.get8();
                    if (r.eof()) return fail(KGK_ERR_PARSE, where + "file too short");
                    if (count >= 128) {
                        count = count == 128 ? (int)r.be16() : count - 127;
                        if (count > left) return fail(KGK_ERR_PARSE, where + "scanline overrun");
                        uint8_t v[4];
                        if (!readval(pk.channel, v)) return fail(KGK_ERR_PARSE, where + "file too short");
                        for (int i = 0; i < count; ++i, dest += 4) copyval(pk.channel, dest, v);
                    } else {
                        ++count;
                        if (count > left) return fail(KGK_ERR_PARSE, where + "scanline overrun");
                        for (int i = 0; i < count; ++i, dest += 4)
                            if (!readval(pk.channel, dest)) return fail(KGK_ERR_PARSE, where + "file too short");
                    }
                    left -= count;
                }
            } else {
                return fail(KGK_ERR_UNSUPPORTED, where + "packet compression type");
            }
        }
    }
    const size_t count = (size_t)w * h;
    pix.resize(count * comp);
    for (size_t i = 0; i < count; ++i) memcpy(&pix[i * comp], &rgba[i * 4], comp);
    *w_out = (int)w;
    *h_out = (int)h;
    *n_out = comp;
    return KGK_OK;
}

// ---------------------------------------------------------------------------
// TGA (stb_image.h:5660-5994); tested last, as stb does
// ---------------------------------------------------------------------------
namespace {
// channels for a pixel / palette entry size (stbi__tga_get_comp)
int tga_comp(int bits, bool grey, bool *rgb16) {
    if (rgb16) *rgb16 = false;
    switch (bits) {
        case 8:
            return 1;
        case 16:
            if (grey) return 2;
            [[fallthrough]];
        case 15:
            if (rgb16) *rgb16 = true;
            return 3;
        case 24:
        case 32:
            return bits / 8;
        default:
            return 0;
    }
}
}  // namespace

bool is_tga(const std::vector<uint8_t> &f) {
    Rd r(f);
    r.get8();
    const int color_type = r.get8();
    if (color_type > 1) return false;
    int sz = r.get8();
    if (color_type == 1) {
        if (sz != 1 && sz != 9) return false;
        r.skip(4);
        sz = r.get8();
        if (sz != 8 && sz != 15 && sz != 16 && sz != 24 && sz != 32) return false;
        r.skip(4);
    } else {
        if (sz != 2 && sz != 3 && sz != 10 && sz != 11) return false;
        r.skip(9);
    }
    if (r.le16() < 1 || r.le16() < 1) return false;
    sz = r.get8();
    if (color_type == 1 && sz != 8 && sz != 16) return false;
    return sz == 8 || sz == 15 || sz == 16 || sz == 24 || sz == 32;
}

kgk_status decode_tga(const std::vector<uint8_t> &f, int *w_out, int *h_out, int *n_out, std::vector<uint8_t> &pix,
                      const char *path) {
    const std::string where = std::string("tga ") + path + ": ";
    Rd r(f);
    const int offset = r.get8(), indexed = r.get8();
    int type = r.get8();
    const int pal_start = (int)r.le16(), pal_len = (int)r.le16(), pal_bits = r.get8();
    r.le16();  // x origin
    r.le16();  // y origin
    const int w = (int)r.le16(), h = (int)r.le16(), bpp = r.get8();
    const int desc = r.get8();
    bool rle = false;
    if (type >= 8) {
        type -= 8;
        rle = true;
    }
    const bool inverted = !((desc >> 5) & 1);  // bottom-up rows unless bit 5
    bool rgb16 = false;
    const int comp = indexed ? tga_comp(pal_bits, false, &rgb16) : tga_comp(bpp, type == 3, &rgb16);
    if (!comp) return fail(KGK_ERR_PARSE, where + "pixel format");
    if (too_large((uint32_t)w, (uint32_t)h, (uint32_t)comp)) return fail(KGK_ERR_PARSE, where + "too large");
    pix.assign((size_t)w * h * comp, 0);
    r.skip(offset);
    auto read_rgb16 = [&](uint8_t *out) {
        const uint32_t px = r.le16();
        out[0] = (uint8_t)((((px >> 10) & 31) * 255) / 31);
        out[1] = (uint8_t)((((px >> 5) & 31) * 255) / 31);
        out[2] = (uint8_t)(((px & 31) * 255) / 31);
    };
    if (!indexed && !rle && !rgb16) {
        for (int i = 0; i < h; ++i) {
            const int row = inverted ? h - i - 1 : i;
            r.getn(&pix[(size_t)row * w * comp], (size_t)w * comp);
        }
    } else {
        std::vector<uint8_t> pal;
        if (indexed) {
            if (pal_len == 0) return fail(KGK_ERR_PARSE, where + "empty palette");
            r.skip(pal_start);
            pal.assign((size_t)pal_len * comp, 0);
            if (rgb16) {
                for (int i = 0; i < pal_len; ++i) read_rgb16(&pal[(size_t)i * comp]);
            } else if (!r.getn(pal.data(), pal.size())) {
                return fail(KGK_ERR_PARSE, where + "truncated palette");
            }
        }
        uint8_t raw[4] = {0, 0, 0, 0};
        int rle_count = 0;
        bool repeating = false, read_next = true;
        for (size_t i = 0; i < (size_t)w * h; ++i) {
            if (rle) {
                if (rle_count == 0) {
                    const int cmd = r.get8();
                    rle_count = 1 + (cmd & 127);
                    repeating = cmd >> 7;
                    read_next = true;
                } else if (!repeating) {
                    read_next = true;
                }
            } else {
                read_next = true;
            }
            if (read_next) {
                if (indexed) {
                    int idx = bpp == 8 ? r.get8() : (int)r.le16();
                    if (idx >= pal_len) idx = 0;
                    for (int j = 0; j < comp; ++j) raw[j] = pal[(size_t)idx * comp + j];
                } else if (rgb16) {
                    read_rgb16(raw);
                } else {
                    for (int j = 0; j < comp; ++j) raw[j] = (uint8_t)r.get8();
                }
                read_next = false;
            }
            for (int j = 0; j < comp; ++j) pix[i * comp + j] = raw[j];
            --rle_count;
        }
        if (inverted) {
            const size_t row = (size_t)w * comp;
            std::vector<uint8_t> tmp(row);
            for (int j = 0; j * 2 < h; ++j) {
                uint8_t *a = &pix[(size_t)j * row], *b = &pix[(size_t)(h - 1 - j) * row];
                if (a == b) continue;
                memcpy(tmp.data(), a, row);
                memcpy(a, b, row);
                memcpy(b, tmp.data(), row);
            }
        }
    }
    if (comp >= 3 && !rgb16)
        for (size_t i = 0; i < (size_t)w * h; ++i) std::swap(pix[i * comp], pix[i * comp + 2]);
    *w_out = w;
    *h_out = h;
    *n_out = comp;
    return KGK_OK;
}

}  // namespace kgk
