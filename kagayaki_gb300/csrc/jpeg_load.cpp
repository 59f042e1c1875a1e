// jpeg_load.cpp - JPEG decoding for scene loading: the JPEG part of the
// reference's stbi_loadf (FileIO/IO_load_images.cuh:10; stb_image v2.27,
// vendored in external_lib/stb).
//
// A JPEG decoder per ITU T.81 (baseline and extended sequential, and
// progressive, Huffman-coded, 8-bit samples, 1, 3 or 4 components, restart
// intervals), with the arithmetic stb_image uses where the standard leaves
// room, so that the bytes equal stb's:
//   * coefficients are dequantised into 16-bit integers (sequential: as
//     they are decoded; progressive: once all scans are read);
//   * the inverse DCT is the integer "islow" factorisation with 12-bit
//     constants: columns keep 2 extra bits ((x + 512) >> 10; a column whose
//     AC terms are all zero is 4 * DC), rows are rounded by
//     (x + 65536 + (128 << 17)) >> 17 and clamped to 0..255;
//   * chroma upsampling: 1:1 as is; 2:1 horizontally or vertically by the
//     3/4 - 1/4 triangle filter ((3a + b + 2) >> 2, edges copied); 2:1 in
//     both by the separable 3:1 filter ((3 t0 + t1 + 8) >> 4 on column sums
//     t = 3 near + far); other ratios replicate samples;
//   * YCbCr -> RGB in fixed point: y * 2^20 + 2^19 plus chroma times
//     round(c * 4096) * 256 for c = 1.402, -0.71414, -0.34414 (whose product
//     keeps only its upper 16 bits), 1.772, then >> 20 and clamped;
//   * three components named 'R','G','B', or an Adobe transform 0 without
//     JFIF, are RGB; four components are CMYK (Adobe transform 0) or YCCK
//     (transform 2), scaled by K with (t + (t >> 8)) >> 8, t = a * b + 128;
//   * the output has 3 channels (1 for a one-component image).
// Malformed streams are rejected with KGK_ERR_PARSE instead of decoding what
// is there.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "kgk_scene.h"

namespace kgk {
namespace {

constexpr int kNoMarker = 0xff;
constexpr int kMaxDim = 1 << 24;

// natural (row-major) position of the i-th coefficient in zigzag order, with
// 15 extra entries of 63 so that a run past the end stays in the block
struct Zigzag {
    uint8_t at[64 + 15];
    Zigzag() {
        int i = 0;
        for (int s = 0; s < 15; ++s) {  // anti-diagonals x + y = s, alternating direction
            for (int k = 0; k <= s; ++k) {
                const int x = (s & 1) ? s - k : k, y = s - x;
                if (x < 8 && y < 8) at[i++] = (uint8_t)(y * 8 + x);
            }
        }
        for (; i < 64 + 15; ++i) at[i] = 63;
    }
};
const Zigzag kZig;

struct Huff {
    uint8_t size[257];
    uint16_t code[256];
    uint8_t values[256];
    uint32_t maxcode[18];  // (last code of each length + 1), left-aligned to 16 bits
    int delta[17];         // symbol index - code, per length
};

// Canonical Huffman codes from the number of codes of each length.
bool build_huff(Huff &h, const int *count) {
    int k = 0;
    for (int i = 0; i < 16; ++i)
        for (int j = 0; j < count[i]; ++j) {
            if (k >= 256) return false;
            h.size[k++] = (uint8_t)(i + 1);
        }
    h.size[k] = 0;
    unsigned code = 0;
    k = 0;
    for (int j = 1; j <= 16; ++j) {
        h.delta[j] = k - (int)code;
        if (h.size[k] == j) {
            while (h.size[k] == j) h.code[k++] = (uint16_t)code++;
            if (code - 1 >= (1u << j)) return false;
        }
        h.maxcode[j] = code << (16 - j);
        code <<= 1;
    }
    h.maxcode[17] = 0xffffffffu;
    return true;
}

struct Comp {
    int id = 0, h = 1, v = 1, tq = 0, hd = 0, ha = 0, dc_pred = 0;
    int x = 0, y = 0, w2 = 0, h2 = 0, coeff_w = 0;
    std::vector<uint8_t> data;
    std::vector<int16_t> coeff;  // progressive only
};

const uint32_t kMask[17] = {0, 1, 3, 7, 15, 31, 63, 127, 255, 511, 1023, 2047, 4095, 8191, 16383, 32767, 65535};

struct Decoder {
    const uint8_t *p;
    size_t n, pos = 0;
    // entropy-coded data
    uint32_t buf = 0;
    int bits = 0;
    int marker = kNoMarker;  // a marker met inside entropy-coded data
    bool nomore = false;
    // tables and frame
    Huff dc[4], ac[4];
    uint16_t dq[4][64];
    int img_x = 0, img_y = 0, img_n = 0;
    int h_max = 1, v_max = 1, mcu_x = 0, mcu_y = 0;
    Comp comp[4];
    bool progressive = false;
    int spec_start = 0, spec_end = 0, succ_high = 0, succ_low = 0, eob_run = 0;
    bool jfif = false;
    int adobe = -1;  // Adobe APP14 colour transform, -1 = none
    int rgb = 0;     // components named 'R', 'G', 'B' in that order
    int scan_n = 0, order[4] = {0, 0, 0, 0};
    int restart_interval = 0, todo = 0;
    std::string err;

    Decoder(const uint8_t *data, size_t size) : p(data), n(size) {
        memset(dc, 0, sizeof dc);
        memset(ac, 0, sizeof ac);
        memset(dq, 0, sizeof dq);
    }

    bool bad(const char *why) {
        if (err.empty()) err = why;
        return false;
    }
    int get8() { return pos < n ? p[pos++] : 0; }  // reads past the end give 0
    int get16() {
        const int a = get8();
        return (a << 8) | get8();
    }
    bool at_eof() const { return pos >= n; }
    void skip(int k) { pos = k < 0 || pos + (size_t)k > n ? n : pos + (size_t)k; }

    // Appends whole bytes until more than 24 bits are held; a marker (0xff
    // followed by a non-zero byte, after 0xff fill bytes) ends the data and
    // zero bits follow.
    void fill() {
        do {
            unsigned b = nomore ? 0u : (unsigned)get8();
            if (b == 0xffu) {
                int c = get8();
                while (c == 0xff) c = get8();
                if (c != 0) {
                    marker = c;
                    nomore = true;
                    return;
                }
            }
            buf |= b << (24 - bits);
            bits += 8;
        } while (bits <= 24);
    }
    int huff(const Huff &h) {
        if (bits < 16) fill();
        const uint32_t top = buf >> 16;
        int k = 1;
        while (k < 17 && top >= h.maxcode[k]) ++k;
        if (k == 17) {
            bits -= 16;
            return -1;
        }
        if (k > bits) return -1;
        const int c = (int)((buf >> (32 - k)) & kMask[k]) + h.delta[k];
        if (c < 0 || c > 255) return -1;
        bits -= k;
        buf <<= k;
        return h.values[c];
    }
    // receive(n) then extend(): a leading 1 bit is a positive value
    int receive_extend(int s) {
        if (bits < s) fill();
        const uint32_t lead = buf >> 31;
        const uint32_t r = s ? (buf << s) | (buf >> (32 - s)) : buf;
        buf = r & ~kMask[s];
        const int v = (int)(r & kMask[s]);
        bits -= s;
        return lead ? v : v - (int)kMask[s];
    }
    int get_bits(int s) {
        if (bits < s) fill();
        const uint32_t r = s ? (buf << s) | (buf >> (32 - s)) : buf;
        buf = r & ~kMask[s];
        bits -= s;
        return (int)(r & kMask[s]);
    }
    bool get_bit() {
        if (bits < 1) fill();
        const uint32_t r = buf;
        buf <<= 1;
        --bits;
        return (r & 0x80000000u) != 0;
    }

    int get_marker() {
        if (marker != kNoMarker) {
            const int m = marker;
            marker = kNoMarker;
            return m;
        }
        int x = get8();
        if (x != 0xff) return kNoMarker;
        while (x == 0xff) x = get8();
        return x;
    }
    void reset() {
        bits = 0;
        buf = 0;
        nomore = false;
        for (Comp &c : comp) c.dc_pred = 0;
        marker = kNoMarker;
        todo = restart_interval ? restart_interval : 0x7fffffff;
        eob_run = 0;
    }

    bool process_marker(int m);
    bool frame_header();
    bool scan_header();
    bool block(int16_t *d, int ci);
    bool block_prog_dc(int16_t *d, int ci);
    bool block_prog_ac(int16_t *d, int ci);
    bool entropy_data();
    bool decode();
};

bool Decoder::process_marker(int m) {
    if (m == kNoMarker) return bad("expected marker");
    if (m == 0xdd) {  // DRI
        if (get16() != 4) return bad("bad DRI length");
        restart_interval = get16();
        return true;
    }
    if (m == 0xdb) {  // DQT
        int L = get16() - 2;
        while (L > 0) {
            const int q = get8();
            const int prec = q >> 4, t = q & 15;
            if (prec != 0 && prec != 1) return bad("bad DQT precision");
            if (t > 3) return bad("bad DQT table");
            for (int i = 0; i < 64; ++i) dq[t][kZig.at[i]] = (uint16_t)(prec ? get16() : get8());
            L -= prec ? 129 : 65;
        }
        return L == 0 || bad("bad DQT length");
    }
    if (m == 0xc4) {  // DHT
        int L = get16() - 2;
        while (L > 0) {
            const int q = get8();
            const int tc = q >> 4, th = q & 15;
            if (tc > 1 || th > 3) return bad("bad DHT header");
            int count[16], total = 0;
            for (int i = 0; i < 16; ++i) total += count[i] = get8();
            L -= 17;
            Huff &h = tc ? ac[th] : dc[th];
            if (!build_huff(h, count)) return bad("bad Huffman code lengths");
            for (int i = 0; i < total; ++i) h.values[i] = (uint8_t)get8();
            L -= total;
        }
        return L == 0 || bad("bad DHT length");
    }
    if ((m >= 0xe0 && m <= 0xef) || m == 0xfe) {  // APPn, COM
        int L = get16();
        if (L < 2) return bad("bad segment length");
        L -= 2;
        if (m == 0xe0 && L >= 5) {
            static const uint8_t tag[5] = {'J', 'F', 'I', 'F', 0};
            bool ok = true;
            for (int i = 0; i < 5; ++i) ok &= get8() == tag[i];
            L -= 5;
            if (ok) jfif = true;
        } else if (m == 0xee && L >= 12) {
            static const uint8_t tag[6] = {'A', 'd', 'o', 'b', 'e', 0};
            bool ok = true;
            for (int i = 0; i < 6; ++i) ok &= get8() == tag[i];
            L -= 6;
            if (ok) {
                get8();   // version
                get16();  // flags
                get16();
                adobe = get8();
                L -= 6;
            }
        }
        skip(L);
        return true;
    }
    return bad("unknown marker");
}

bool Decoder::frame_header() {
    const int Lf = get16();
    if (Lf < 11) return bad("bad SOF length");
    if (get8() != 8) return bad("only 8-bit samples are supported");
    img_y = get16();
    if (img_y == 0) return bad("no height in the frame header");
    img_x = get16();
    if (img_x == 0) return bad("zero width");
    if (img_x > kMaxDim || img_y > kMaxDim) return bad("image too large");
    img_n = get8();
    if (img_n != 1 && img_n != 3 && img_n != 4) return bad("bad component count");
    if (Lf != 8 + 3 * img_n) return bad("bad SOF length");
    rgb = 0;
    static const uint8_t kRGB[3] = {'R', 'G', 'B'};
    for (int i = 0; i < img_n; ++i) {
        Comp &c = comp[i];
        c.id = get8();
        if (img_n == 3 && c.id == kRGB[i]) ++rgb;
        const int q = get8();
        c.h = q >> 4;
        c.v = q & 15;
        if (c.h < 1 || c.h > 4) return bad("bad H");
        if (c.v < 1 || c.v > 4) return bad("bad V");
        c.tq = get8();
        if (c.tq > 3) return bad("bad TQ");
    }
    if ((int64_t)img_x * img_y * img_n > (int64_t)0x7fffffff) return bad("image too large");
    h_max = v_max = 1;
    for (int i = 0; i < img_n; ++i) {
        h_max = std::max(h_max, comp[i].h);
        v_max = std::max(v_max, comp[i].v);
    }
    for (int i = 0; i < img_n; ++i)
        if (h_max % comp[i].h || v_max % comp[i].v) return bad("fractional sampling ratio");
    mcu_x = (img_x + h_max * 8 - 1) / (h_max * 8);
    mcu_y = (img_y + v_max * 8 - 1) / (v_max * 8);
    for (int i = 0; i < img_n; ++i) {
        Comp &c = comp[i];
        c.x = (img_x * c.h + h_max - 1) / h_max;  // samples of the component
        c.y = (img_y * c.v + v_max - 1) / v_max;
        c.w2 = mcu_x * c.h * 8;                   // padded to whole MCUs
        c.h2 = mcu_y * c.v * 8;
        c.data.assign((size_t)c.w2 * c.h2, 0);
        if (progressive) {
            c.coeff_w = c.w2 / 8;
            c.coeff.assign((size_t)c.w2 * c.h2, 0);
        }
    }
    return true;
}

bool Decoder::scan_header() {
    const int Ls = get16();
    scan_n = get8();
    if (scan_n < 1 || scan_n > 4 || scan_n > img_n) return bad("bad SOS component count");
    if (Ls != 6 + 2 * scan_n) return bad("bad SOS length");
    for (int i = 0; i < scan_n; ++i) {
        const int id = get8(), q = get8();
        int which = 0;
        while (which < img_n && comp[which].id != id) ++which;
        if (which == img_n) return bad("SOS names an unknown component");
        comp[which].hd = q >> 4;
        comp[which].ha = q & 15;
        if (comp[which].hd > 3 || comp[which].ha > 3) return bad("bad Huffman table index");
        order[i] = which;
    }
    spec_start = get8();
    spec_end = get8();
    const int aa = get8();
    succ_high = aa >> 4;
    succ_low = aa & 15;
    if (progressive) {
        if (spec_start > 63 || spec_end > 63 || spec_start > spec_end || succ_high > 13 || succ_low > 13)
            return bad("bad SOS");
    } else {
        if (spec_start != 0 || succ_high != 0 || succ_low != 0) return bad("bad SOS");
        spec_end = 63;
    }
    return true;
}

// One sequential block: DC difference, AC run/size codes, dequantised.
bool Decoder::block(int16_t *d, int ci) {
    Comp &c = comp[ci];
    if (bits < 16) fill();
    const int t = huff(dc[c.hd]);
    if (t < 0 || t > 15) return bad("bad Huffman code");
    memset(d, 0, 64 * sizeof(int16_t));
    const int diff = t ? receive_extend(t) : 0;
    const int dcv = c.dc_pred + diff;
    c.dc_pred = dcv;
    const uint16_t *q = dq[c.tq];
    d[0] = (int16_t)(dcv * q[0]);
    int k = 1;
    do {
        const int rs = huff(ac[c.ha]);
        if (rs < 0) return bad("bad Huffman code");
        const int s = rs & 15, r = rs >> 4;
        if (s == 0) {
            if (rs != 0xf0) break;  // end of block
            k += 16;
        } else {
            k += r;
            const int z = kZig.at[k++];
            d[z] = (int16_t)(receive_extend(s) * q[z]);
        }
    } while (k < 64);
    return true;
}

bool Decoder::block_prog_dc(int16_t *d, int ci) {
    Comp &c = comp[ci];
    if (spec_end != 0) return bad("DC scan with AC coefficients");
    if (bits < 16) fill();
    if (succ_high == 0) {  // first DC scan
        memset(d, 0, 64 * sizeof(int16_t));
        const int t = huff(dc[c.hd]);
        if (t < 0 || t > 15) return bad("bad Huffman code");
        const int diff = t ? receive_extend(t) : 0;
        const int dcv = c.dc_pred + diff;
        c.dc_pred = dcv;
        d[0] = (int16_t)(dcv * (1 << succ_low));
    } else if (get_bit()) {  // refinement: one more bit
        d[0] = (int16_t)(d[0] + (1 << succ_low));
    }
    return true;
}

bool Decoder::block_prog_ac(int16_t *d, int ci) {
    Comp &c = comp[ci];
    if (spec_start == 0) return bad("AC scan with the DC coefficient");
    if (succ_high == 0) {  // first AC scan of the band
        const int shift = succ_low;
        if (eob_run) {
            --eob_run;
            return true;
        }
        int k = spec_start;
        do {
            const int rs = huff(ac[c.ha]);
            if (rs < 0) return bad("bad Huffman code");
            const int s = rs & 15, r = rs >> 4;
            if (s == 0) {
                if (r < 15) {  // end-of-band run of 2^r (+ r more bits) blocks
                    eob_run = 1 << r;
                    if (r) eob_run += get_bits(r);
                    --eob_run;
                    break;
                }
                k += 16;
            } else {
                k += r;
                const int z = kZig.at[k++];
                d[z] = (int16_t)(receive_extend(s) * (1 << shift));
            }
        } while (k <= spec_end);
        return true;
    }
    // refinement scan: one correction bit per nonzero coefficient met, and
    // newly nonzero coefficients of magnitude 1 << succ_low
    const int16_t bit = (int16_t)(1 << succ_low);
    auto refine = [&](int16_t *q) {
        if (get_bit() && (*q & bit) == 0) *q = (int16_t)(*q > 0 ? *q + bit : *q - bit);
    };
    if (eob_run) {
        --eob_run;
        for (int k = spec_start; k <= spec_end; ++k) {
            int16_t *q = &d[kZig.at[k]];
            if (*q != 0) refine(q);
        }
        return true;
    }
    int k = spec_start;
    do {
        const int rs = huff(ac[c.ha]);
        if (rs < 0) return bad("bad Huffman code");
        int s = rs & 15, r = rs >> 4;
        if (s == 0) {
            if (r < 15) {
                eob_run = (1 << r) - 1;
                if (r) eob_run += get_bits(r);
                r = 64;  // the rest of the band only refines
            }
            // r == 15: a run of 16 zero coefficients, value 0
        } else {
            if (s != 1) return bad("bad refinement code");
            s = get_bit() ? bit : -bit;
        }
        while (k <= spec_end) {
            int16_t *q = &d[kZig.at[k++]];
            if (*q != 0) {
                refine(q);
            } else {
                if (r == 0) {
                    *q = (int16_t)s;
                    break;
                }
                --r;
            }
        }
    } while (k <= spec_end);
    return true;
}

// Integer inverse DCT of one 8x8 block into out (stride bytes per row).  The
// published method is the Independent JPEG Group's "islow" separable integer
// IDCT (jidctint.c, after Loeffler, Ligtenberg and Moschytz 1989) with 12-bit
// fixed-point constants, in the variant stb_image v2.27 uses (columns first,
// its rounding biases and shifts), which every output bit of stbi_loadf
// depends on.
constexpr int fix12(double x) { return (int)(x * 4096 + 0.5); }

struct Idct1 {
    int t0, t1, t2, t3, x0, x1, x2, x3;
};

inline Idct1 idct_1d(int s0, int s1, int s2, int s3, int s4, int s5, int s6, int s7) {
    Idct1 r;
    int p2 = s2, p3 = s6;
    int p1 = (p2 + p3) * fix12(0.5411961f);
    r.t2 = p1 + p3 * fix12(-1.847759065f);
    r.t3 = p1 + p2 * fix12(0.765366865f);
    p2 = s0;
    p3 = s4;
    r.t0 = (p2 + p3) * 4096;
    r.t1 = (p2 - p3) * 4096;
    r.x0 = r.t0 + r.t3;
    r.x3 = r.t0 - r.t3;
    r.x1 = r.t1 + r.t2;
    r.x2 = r.t1 - r.t2;
    int t0 = s7, t1 = s5, t2 = s3, t3 = s1;
    p3 = t0 + t2;
    int p4 = t1 + t3;
    p1 = t0 + t3;
    p2 = t1 + t2;
    const int p5 = (p3 + p4) * fix12(1.175875602f);
    t0 = t0 * fix12(0.298631336f);
    t1 = t1 * fix12(2.053119869f);
    t2 = t2 * fix12(3.072711026f);
    t3 = t3 * fix12(1.501321110f);
    p1 = p5 + p1 * fix12(-0.899976223f);
    p2 = p5 + p2 * fix12(-2.562915447f);
    p3 = p3 * fix12(-1.961570560f);
    p4 = p4 * fix12(-0.390180644f);
    r.t3 = t3 + p1 + p4;
    r.t2 = t2 + p2 + p3;
    r.t1 = t1 + p2 + p4;
    r.t0 = t0 + p1 + p3;
    return r;
}

inline uint8_t clamp255(int x) { return (uint8_t)(x < 0 ? 0 : (x > 255 ? 255 : x)); }

void idct_block(uint8_t *out, int stride, const int16_t *d) {
    int v[64];
    for (int i = 0; i < 8; ++i) {
        const int16_t *c = d + i;
        if (!c[8] && !c[16] && !c[24] && !c[32] && !c[40] && !c[48] && !c[56]) {
            const int dcterm = c[0] * 4;
            for (int k = 0; k < 8; ++k) v[i + 8 * k] = dcterm;
            continue;
        }
        Idct1 r = idct_1d(c[0], c[8], c[16], c[24], c[32], c[40], c[48], c[56]);
        r.x0 += 512;
        r.x1 += 512;
        r.x2 += 512;
        r.x3 += 512;
        v[i] = (r.x0 + r.t3) >> 10;
        v[i + 56] = (r.x0 - r.t3) >> 10;
        v[i + 8] = (r.x1 + r.t2) >> 10;
        v[i + 48] = (r.x1 - r.t2) >> 10;
        v[i + 16] = (r.x2 + r.t1) >> 10;
        v[i + 40] = (r.x2 - r.t1) >> 10;
        v[i + 24] = (r.x3 + r.t0) >> 10;
        v[i + 32] = (r.x3 - r.t0) >> 10;
    }
    for (int i = 0; i < 8; ++i) {
        const int *w = v + 8 * i;
        uint8_t *o = out + (size_t)i * stride;
        Idct1 r = idct_1d(w[0], w[1], w[2], w[3], w[4], w[5], w[6], w[7]);
        const int bias = 65536 + (128 << 17);
        r.x0 += bias;
        r.x1 += bias;
        r.x2 += bias;
        r.x3 += bias;
        o[0] = clamp255((r.x0 + r.t3) >> 17);
        o[7] = clamp255((r.x0 - r.t3) >> 17);
        o[1] = clamp255((r.x1 + r.t2) >> 17);
        o[6] = clamp255((r.x1 - r.t2) >> 17);
        o[2] = clamp255((r.x2 + r.t1) >> 17);
        o[5] = clamp255((r.x2 - r.t1) >> 17);
        o[3] = clamp255((r.x3 + r.t0) >> 17);
        o[4] = clamp255((r.x3 - r.t0) >> 17);
    }
}

bool Decoder::entropy_data() {
    reset();
    int16_t blk[64];
    // counts down the restart interval after each MCU; false ends the scan
    auto next_mcu = [&]() {
        if (--todo > 0) return true;
        if (bits < 24) fill();
        if (marker < 0xd0 || marker > 0xd7) return false;  // not a restart marker: stop here
        reset();
        return true;
    };
    if (scan_n == 1) {  // non-interleaved: the component's own blocks in raster order
        const int ci = order[0];
        Comp &c = comp[ci];
        const int w = (c.x + 7) >> 3, h = (c.y + 7) >> 3;
        for (int j = 0; j < h; ++j)
            for (int i = 0; i < w; ++i) {
                if (!progressive) {
                    if (!block(blk, ci)) return false;
                    idct_block(c.data.data() + (size_t)c.w2 * j * 8 + i * 8, c.w2, blk);
                } else {
                    int16_t *d = c.coeff.data() + 64 * ((size_t)i + (size_t)j * c.coeff_w);
                    if (!(spec_start == 0 ? block_prog_dc(d, ci) : block_prog_ac(d, ci))) return false;
                }
                if (!next_mcu()) return true;
            }
        return true;
    }
    for (int j = 0; j < mcu_y; ++j)
        for (int i = 0; i < mcu_x; ++i) {
            for (int k = 0; k < scan_n; ++k) {
                const int ci = order[k];
                Comp &c = comp[ci];
                for (int y = 0; y < c.v; ++y)
                    for (int x = 0; x < c.h; ++x) {
                        const int bx = i * c.h + x, by = j * c.v + y;
                        if (!progressive) {
                            if (!block(blk, ci)) return false;
                            idct_block(c.data.data() + (size_t)c.w2 * by * 8 + bx * 8, c.w2, blk);
                        } else {
                            int16_t *d = c.coeff.data() + 64 * ((size_t)bx + (size_t)by * c.coeff_w);
                            if (!block_prog_dc(d, ci)) return false;  // interleaved progressive scans are DC scans
                        }
                    }
            }
            if (!next_mcu()) return true;
        }
    return true;
}

bool Decoder::decode() {
    int m = get_marker();
    if (m != 0xd8) return bad("no SOI marker");
    m = get_marker();
    while (m != 0xc0 && m != 0xc1 && m != 0xc2) {
        if (!process_marker(m)) return false;
        m = get_marker();
        while (m == kNoMarker) {  // padding between segments
            if (at_eof()) return bad("no SOF marker");
            m = get_marker();
        }
    }
    progressive = m == 0xc2;
    if (!frame_header()) return false;
    m = get_marker();
    while (m != 0xd9) {  // until EOI
        if (m == 0xda) {  // SOS
            if (!scan_header() || !entropy_data()) return false;
            if (marker == kNoMarker) {  // zero bytes after the data: look for the next marker
                while (!at_eof()) {
                    if (get8() == 255) {
                        marker = get8();
                        break;
                    }
                }
            }
        } else if (m == 0xdc) {  // DNL
            const int Ld = get16(), NL = get16();
            if (Ld != 4) return bad("bad DNL length");
            if (NL != img_y) return bad("bad DNL height");
        } else if (!process_marker(m)) {
            return false;
        }
        m = get_marker();
    }
    if (progressive) {  // dequantise and transform the accumulated coefficients
        for (int ci = 0; ci < img_n; ++ci) {
            Comp &c = comp[ci];
            const int w = (c.x + 7) >> 3, h = (c.y + 7) >> 3;
            for (int j = 0; j < h; ++j)
                for (int i = 0; i < w; ++i) {
                    int16_t *d = c.coeff.data() + 64 * ((size_t)i + (size_t)j * c.coeff_w);
                    for (int k = 0; k < 64; ++k) d[k] = (int16_t)(d[k] * dq[c.tq][k]);
                    idct_block(c.data.data() + (size_t)c.w2 * j * 8 + i * 8, c.w2, d);
                }
        }
    }
    return true;
}

// Row upsamplers: w input samples -> the expanded row (see the file comment).
const uint8_t *up_1(uint8_t *, const uint8_t *near, const uint8_t *, int, int) { return near; }

const uint8_t *up_v2(uint8_t *out, const uint8_t *near, const uint8_t *far, int w, int) {
    for (int i = 0; i < w; ++i) out[i] = (uint8_t)((3 * near[i] + far[i] + 2) >> 2);
    return out;
}

const uint8_t *up_h2(uint8_t *out, const uint8_t *in, const uint8_t *, int w, int) {
    if (w == 1) {
        out[0] = out[1] = in[0];
        return out;
    }
    out[0] = in[0];
    out[1] = (uint8_t)((in[0] * 3 + in[1] + 2) >> 2);
    int i = 1;
    for (; i < w - 1; ++i) {
        const int c = 3 * in[i] + 2;
        out[2 * i] = (uint8_t)((c + in[i - 1]) >> 2);
        out[2 * i + 1] = (uint8_t)((c + in[i + 1]) >> 2);
    }
    out[2 * i] = (uint8_t)((in[w - 2] * 3 + in[w - 1] + 2) >> 2);
    out[2 * i + 1] = in[w - 1];
    return out;
}

const uint8_t *up_hv2(uint8_t *out, const uint8_t *near, const uint8_t *far, int w, int) {
    if (w == 1) {
        out[0] = out[1] = (uint8_t)((3 * near[0] + far[0] + 2) >> 2);
        return out;
    }
    int t1 = 3 * near[0] + far[0];
    out[0] = (uint8_t)((t1 + 2) >> 2);
    for (int i = 1; i < w; ++i) {
        const int t0 = t1;
        t1 = 3 * near[i] + far[i];
        out[2 * i - 1] = (uint8_t)((3 * t0 + t1 + 8) >> 4);
        out[2 * i] = (uint8_t)((3 * t1 + t0 + 8) >> 4);
    }
    out[2 * w - 1] = (uint8_t)((t1 + 2) >> 2);
    return out;
}

const uint8_t *up_generic(uint8_t *out, const uint8_t *near, const uint8_t *, int w, int hs) {
    for (int i = 0; i < w; ++i)
        for (int j = 0; j < hs; ++j) out[i * hs + j] = near[i];
    return out;
}

inline uint8_t clamp_shift20(int x) {
    x >>= 20;
    return (uint8_t)(x < 0 ? 0 : (x > 255 ? 255 : x));
}

constexpr int fix20(float x) { return ((int)(x * 4096.0f + 0.5f)) << 8; }

void ycbcr_to_rgb(uint8_t *out, const uint8_t *y, const uint8_t *cb, const uint8_t *cr, int count, int step) {
    for (int i = 0; i < count; ++i, out += step) {
        const int yf = (y[i] << 20) + (1 << 19);
        const int crv = cr[i] - 128, cbv = cb[i] - 128;
        const int gcb = (int)((uint32_t)(cbv * -fix20(0.34414f)) & 0xffff0000u);
        out[0] = clamp_shift20(yf + crv * fix20(1.40200f));
        out[1] = clamp_shift20(yf + crv * -fix20(0.71414f) + gcb);
        out[2] = clamp_shift20(yf + cbv * fix20(1.77200f));
    }
}

inline uint8_t scale_by(uint8_t x, uint8_t y) {
    const unsigned t = (unsigned)x * y + 128;
    return (uint8_t)((t + (t >> 8)) >> 8);
}

}  // namespace

kgk_status decode_jpeg(const std::vector<uint8_t> &f, int *w_out, int *h_out, int *n_out, std::vector<uint8_t> &pix,
                       const char *path) {
    Decoder z(f.data(), f.size());
    if (!z.decode()) return fail(KGK_ERR_PARSE, std::string("JPEG: ") + z.err + ": " + path);
    const int W = z.img_x, H = z.img_y;
    const int n = z.img_n >= 3 ? 3 : 1;
    const bool is_rgb = z.img_n == 3 && (z.rgb == 3 || (z.adobe == 0 && !z.jfif));
    typedef const uint8_t *(*Up)(uint8_t *, const uint8_t *, const uint8_t *, int, int);
    struct Row {
        Up up;
        const uint8_t *line0, *line1;
        int hs, vs, w_lores, ystep, ypos;
        std::vector<uint8_t> buf;
    } rows[4];
    for (int k = 0; k < z.img_n; ++k) {
        Row &r = rows[k];
        r.hs = z.h_max / z.comp[k].h;
        r.vs = z.v_max / z.comp[k].v;
        r.ystep = r.vs >> 1;
        r.w_lores = (W + r.hs - 1) / r.hs;
        r.ypos = 0;
        r.line0 = r.line1 = z.comp[k].data.data();
        r.buf.assign((size_t)W + 3, 0);
        r.up = (r.hs == 1 && r.vs == 1)   ? up_1
               : (r.hs == 1 && r.vs == 2) ? up_v2
               : (r.hs == 2 && r.vs == 1) ? up_h2
               : (r.hs == 2 && r.vs == 2) ? up_hv2
                                          : up_generic;
    }
    pix.assign((size_t)W * H * n, 0);
    const uint8_t *co[4] = {nullptr, nullptr, nullptr, nullptr};
    for (int j = 0; j < H; ++j) {
        uint8_t *out = pix.data() + (size_t)n * W * j;
        for (int k = 0; k < z.img_n; ++k) {
            Row &r = rows[k];
            // the two source rows nearest to this output row: vertical weight 3:1
            const bool bottom = r.ystep >= (r.vs >> 1);
            co[k] = r.up(r.buf.data(), bottom ? r.line1 : r.line0, bottom ? r.line0 : r.line1, r.w_lores, r.hs);
            if (++r.ystep >= r.vs) {
                r.ystep = 0;
                r.line0 = r.line1;
                if (++r.ypos < z.comp[k].y) r.line1 += z.comp[k].w2;
            }
        }
        if (n == 1) {
            memcpy(out, co[0], (size_t)W);
        } else if (z.img_n == 3) {
            if (is_rgb) {
                for (int i = 0; i < W; ++i) {
                    out[3 * i] = co[0][i];
                    out[3 * i + 1] = co[1][i];
                    out[3 * i + 2] = co[2][i];
                }
            } else {
                ycbcr_to_rgb(out, co[0], co[1], co[2], W, 3);
            }
        } else if (z.adobe == 0) {  // CMYK
            for (int i = 0; i < W; ++i) {
                const uint8_t m = co[3][i];
                for (int c = 0; c < 3; ++c) out[3 * i + c] = scale_by(co[c][i], m);
            }
        } else if (z.adobe == 2) {  // YCCK
            ycbcr_to_rgb(out, co[0], co[1], co[2], W, 3);
            for (int i = 0; i < W; ++i) {
                const uint8_t m = co[3][i];
                for (int c = 0; c < 3; ++c) out[3 * i + c] = scale_by((uint8_t)(255 - out[3 * i + c]), m);
            }
        } else {  // YCbCr with a fourth channel, which is ignored
            ycbcr_to_rgb(out, co[0], co[1], co[2], W, 3);
        }
    }
    *w_out = W;
    *h_out = H;
    *n_out = n;
    return KGK_OK;
}

}  // namespace kgk
