// obj_load.cpp - Wavefront OBJ / MTL scene loading (replaces load_object,
// FileIO/IO_load_WavefrontObj.cuh:10-127, and load_HDR / load_Textures,
// FileIO/IO_load_images.cuh:9-29).
//
// The reference parses with tinyobjloader v2.0.0rc10 (vendored,
// external_lib/tinyobjloader; config: triangulate, "simple" triangulation) and
// turns every triangle of every shape into a Triangle record.  This file
// restates the parts of that library's published behaviour the render path
// depends on:
//   * numbers: decimal mantissa accumulated in double (fraction digits add
//     d * 10^-k), exponent applied as ldexp(m * 5^e, e), then cast to float;
//   * indices: 1-based, negative = relative to the current count, 0 = error;
//   * shapes: a new shape starts at every `g` / `o` line (when the current one
//     has faces); `usemtl` changes the material of the following faces only;
//   * triangulation: triangles as given; quads split along the shorter
//     diagonal; larger polygons by the library's ear clipping in the plane of
//     the two axes with the largest corner cross product;
//   * smoothing groups: `s off` / `s 0` = flat, `s N` = smooth;
//   * MTL: Kd, Ks, Ke, Ni, Pr, Pm, map_Kd (Kd defaults to 0.6 when map_Kd
//     comes before any Kd line of the file); unknown keys are ignored.
// Then the reference's own conversion (IO_load_WavefrontObj.cuh:32-127):
//   material id = usemtl index + 1 (0 = the reserved grey material,
//   scene.cuh:14-18); normals normalised ((10000,0,0) for a zero normal);
//   texcoords (u, v, 0); diffuse + 1e-4 when a component is 0; Lambert;
//   specular = |Ks|; textured and untextured materials take the two parameter
//   sets of IO_load_WavefrontObj.cuh:114-122; texture pixels + 1e-4.
// Differences by design: vertices without vn (or with an index past the vn
// records) take the face's geometric normal and without vt take (0, 0, 0)
// (the reference indexes missing entries); MTL
// files and textures are looked up in the OBJ file's directory (the reference
// uses the working directory); malformed input returns an error instead of
// exiting.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <map>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "kgk_scene.h"

using namespace kgk;

namespace kgk {
kgk_status load_image_float(const char *path, kgk_texture *out);
}

namespace {

inline bool is_space(char c) { return c == ' ' || c == '\t'; }
inline bool is_digit(char c) { return (unsigned)(c - '0') < 10u; }
inline bool is_newline(char c) { return c == '\r' || c == '\n' || c == '\0'; }

// 10^-k as the fraction digits of tinyobjloader's reader weigh them: the
// nearest double for k < 8, std::pow beyond.
double fraction_weight(int k) {
    static const double w[8] = {1.0, 1e-1, 1e-2, 1e-3, 1e-4, 1e-5, 1e-6, 1e-7};
    return k < 8 ? w[k] : std::pow(10.0, -k);
}

// A number as tinyobjloader v2.0.0rc10 reads one from [s, end):
//   [+|-] ( digits [ '.' digits* ] | '.' digits* ) [ (e|E) [+|-] digits ]
// The value is accumulated in double: integer digits as m = 10 m + d, the
// k-th fraction digit adds d * 10^-k, and an exponent e != 0 scales by
// ldexp(m * 5^e, e), and the sign multiplies the result.  Reading stops at the first character outside the
// grammar (the value read so far stands), but an exponent marker must be
// followed by digits, and an exponent above INT_MAX is rejected.  `end` must
// point at a non-digit character (the callers end tokens at blanks).
bool parse_double(const char *s, const char *end, double *out) {
    const char *c = s;
    auto here = [&](char a, char b) { return c != end && (*c == a || *c == b); };
    auto digit_here = [&]() { return c != end && is_digit(*c); };
    if (c == end || !(here('+', '-') || is_digit(*c) || *c == '.')) return false;
    const bool negative = *c == '-';
    if (here('+', '-')) ++c;
    double m = 0.0;
    if (!here('.', '.')) {  // an integer part is required unless a '.' leads
        const char *first = c;
        for (; digit_here(); ++c) m = m * 10 + (*c - '0');
        if (c == first) return false;
    }
    if (here('.', '.')) {
        ++c;
        for (int k = 1; digit_here(); ++c, ++k) m += (double)(*c - '0') * fraction_weight(k);
    }
    int e = 0;
    if (here('e', 'E')) {
        ++c;
        const bool e_negative = here('-', '-');
        if (here('+', '-')) ++c;
        const char *first = c;
        for (; digit_here(); ++c) {
            if (e > 2147483647 / 10) return false;
            e = e * 10 + (*c - '0');
        }
        if (c == first) return false;
        if (e_negative) e = -e;
    }
    const double v = e != 0 ? std::ldexp(m * std::pow(5.0, e), e) : m;
    // The sign is a factor, multiplied in: a NaN (0 * 5^e with 5^e overflowing)
    // then keeps the sign bit the hardware gave it, where a negation would
    // flip it.  Loaded from a table so the compiler keeps the multiplication.
    static const double kSign[2] = {1.0, -1.0};
    *out = kSign[negative] * v;
    return true;
}

// Token readers: a token ends at space, tab or '\r'.
float read_real(const char **t, double dflt = 0.0) {
    *t += strspn(*t, " \t");
    const char *end = *t + strcspn(*t, " \t\r");
    double v = dflt;
    parse_double(*t, end, &v);
    *t = end;
    return (float)v;
}
std::string read_string(const char **t) {
    *t += strspn(*t, " \t");
    const size_t e = strcspn(*t, " \t\r");
    std::string s(*t, *t + e);
    *t += e;
    return s;
}

struct VIdx {
    int v = -1, vt = -1, vn = -1;
};

// 1-based / negative-relative index; 0 is an error for v, allowed (as -1) for vt / vn.
bool fix_index(int idx, int n, int *out, bool allow_zero) {
    if (idx > 0) { *out = idx - 1; return true; }
    if (idx == 0) { *out = -1; return allow_zero; }
    *out = n + idx;
    return true;
}

bool parse_triple(const char **t, int nv, int nvn, int nvt, VIdx *r) {
    VIdx vi;
    if (!fix_index(atoi(*t), nv, &vi.v, false)) return false;
    *t += strcspn(*t, "/ \t\r");
    if ((*t)[0] != '/') { *r = vi; return true; }
    ++*t;
    if ((*t)[0] == '/') {
        ++*t;
        if (!fix_index(atoi(*t), nvn, &vi.vn, true)) return false;
        *t += strcspn(*t, "/ \t\r");
        *r = vi;
        return true;
    }
    if (!fix_index(atoi(*t), nvt, &vi.vt, true)) return false;
    *t += strcspn(*t, "/ \t\r");
    if ((*t)[0] != '/') { *r = vi; return true; }
    ++*t;
    if (!fix_index(atoi(*t), nvn, &vi.vn, true)) return false;
    *t += strcspn(*t, "/ \t\r");
    *r = vi;
    return true;
}

struct Tri {
    VIdx a, b, c;
    int mat;
    unsigned smooth;
};
struct Shape {
    std::vector<Tri> tris;
    bool other_prims = false;  // lines / points (no triangles, but the shape counts)
};

struct MtlMaterial {
    std::string name;
    float diffuse[3] = {0, 0, 0}, specular[3] = {0, 0, 0}, emission[3] = {0, 0, 0};
    float ior = 1.0f, roughness = 0.0f, metallic = 0.0f;
    // PBR extension (Pr / Pm above, and Ps, Pc, Pcr, aniso): read for the
    // Disney mapping only; has_pbr = any of Pr, Pm, Ps, Pc, Pcr, aniso given
    float sheen = 0.0f, clearcoat = 0.0f, clearcoat_roughness = 0.0f, anisotropy = 0.0f;
    bool has_pbr = false, has_ni = false;
    std::string diffuse_tex;
};

// One line at a time: '\n', '\r\n' or '\r' ends a line.
struct Lines {
    const std::string &s;
    size_t pos = 0;
    bool next(std::string &line) {
        if (pos >= s.size()) return false;
        line.clear();
        while (pos < s.size()) {
            const char c = s[pos++];
            if (c == '\n') break;
            if (c == '\r') {
                if (pos < s.size() && s[pos] == '\n') ++pos;
                break;
            }
            line += c;
        }
        return true;
    }
};

bool read_text(const std::string &path, std::string &out) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return false;
    // one read of the whole file when its size is known, then whatever follows
    if (fseek(f, 0, SEEK_END) == 0) {
        const long size = ftell(f);
        if (size > 0 && fseek(f, 0, SEEK_SET) == 0) {
            out.resize((size_t)size);
            out.resize(fread(&out[0], 1, (size_t)size, f));
        } else {
            fseek(f, 0, SEEK_SET);
        }
    }
    char buf[1 << 16];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, n);
    fclose(f);
    return true;
}

// tinyobjloader's LoadMtl.
void parse_mtl(const std::string &text, std::vector<MtlMaterial> &mats, std::map<std::string, int> &by_name) {
    MtlMaterial m;
    bool has_kd = false;
    Lines lines{text};
    std::string ln;
    auto flush = [&]() {
        by_name.insert({m.name, (int)mats.size()});
        mats.push_back(m);
    };
    while (lines.next(ln)) {
        if (!ln.empty()) ln = ln.substr(0, ln.find_last_not_of(" \t") + 1);
        if (!ln.empty() && ln.back() == '\n') ln.pop_back();
        if (!ln.empty() && ln.back() == '\r') ln.pop_back();
        if (ln.empty()) continue;
        const char *t = ln.c_str();
        t += strspn(t, " \t");
        if (t[0] == '\0' || t[0] == '#') continue;
        if (!strncmp(t, "newmtl", 6) && is_space(t[6])) {
            if (!m.name.empty()) flush();
            m = MtlMaterial();  // has_kd carries over, as in tinyobjloader
            m.name = std::string(t + 7);
            continue;
        }
        auto rgb = [&](float *dst) {
            t += 2;
            const float r = read_real(&t), g = read_real(&t), b = read_real(&t);
            dst[0] = r;
            dst[1] = g;
            dst[2] = b;
        };
        if (t[0] == 'K' && t[1] == 'd' && is_space(t[2])) { rgb(m.diffuse); has_kd = true; continue; }
        if (t[0] == 'K' && t[1] == 's' && is_space(t[2])) { rgb(m.specular); continue; }
        if (t[0] == 'K' && t[1] == 'e' && is_space(t[2])) { rgb(m.emission); continue; }
        if (t[0] == 'N' && t[1] == 'i' && is_space(t[2])) { t += 2; m.ior = read_real(&t); m.has_ni = true; continue; }
        if (t[0] == 'P' && t[1] == 'r' && is_space(t[2])) { t += 2; m.roughness = read_real(&t); m.has_pbr = true; continue; }
        if (t[0] == 'P' && t[1] == 'm' && is_space(t[2])) { t += 2; m.metallic = read_real(&t); m.has_pbr = true; continue; }
        if (t[0] == 'P' && t[1] == 's' && is_space(t[2])) { t += 2; m.sheen = read_real(&t); m.has_pbr = true; continue; }
        if (t[0] == 'P' && t[1] == 'c' && is_space(t[2])) { t += 2; m.clearcoat = read_real(&t); m.has_pbr = true; continue; }
        if (!strncmp(t, "Pcr", 3) && is_space(t[3])) {
            t += 3;
            m.clearcoat_roughness = read_real(&t);
            m.has_pbr = true;
            continue;
        }
        if (!strncmp(t, "aniso", 5) && is_space(t[5])) {
            t += 5;
            m.anisotropy = read_real(&t);
            m.has_pbr = true;
            continue;
        }
        if (!strncmp(t, "map_Kd", 6) && is_space(t[6])) {
            t += 7;
            // texture options (-name values) precede the file name, which runs to the line end
            std::string name;
            while (!is_newline(*t)) {
                t += strspn(t, " \t");
                if (*t == '-') {
                    // skip an option and its numeric / on|off arguments
                    t += strcspn(t, " \t\r");
                    for (;;) {
                        const char *u = t + strspn(t, " \t");
                        const char *e = u + strcspn(u, " \t\r");
                        double d;
                        const bool num = parse_double(u, e, &d) && e > u;
                        const bool onoff = (e - u == 2 && !strncmp(u, "on", 2)) || (e - u == 3 && !strncmp(u, "off", 3));
                        if (!num && !onoff) break;
                        t = e;
                    }
                } else {
                    name = std::string(t);
                    break;
                }
            }
            m.diffuse_tex = name;
            if (!has_kd) m.diffuse[0] = m.diffuse[1] = m.diffuse[2] = 0.6f;
            continue;
        }
    }
    flush();
}

std::string dir_of(const std::string &path) {
    const size_t k = path.find_last_of("/\\");
    return k == std::string::npos ? std::string() : path.substr(0, k + 1);
}

int pnpoly3(const float *vx, const float *vy, float tx, float ty) {
    int c = 0;
    for (int i = 0, j = 2; i < 3; j = i++) {
        if (((vy[i] > ty) != (vy[j] > ty)) && (tx < (vx[j] - vx[i]) * (ty - vy[i]) / (vy[j] - vy[i]) + vx[i])) c = !c;
    }
    return c;
}

// Emits the triangles of one polygon (tinyobjloader's "simple" triangulation)
// of n corners.  Only the first `vsize` floats of v (the vertices read before
// the polygon's group ended) are visible to it.
void triangulate(const VIdx *fv, size_t n, unsigned smooth, int mat, const std::vector<float> &v, size_t vsize,
                 std::vector<Tri> &out) {
    if (n < 3) return;
    if (n == 3) {
        out.push_back({fv[0], fv[1], fv[2], mat, smooth});
        return;
    }
    auto valid = [&](const VIdx &x) { return x.v >= 0 && (size_t)(3 * x.v + 2) < vsize; };
    if (n == 4) {
        const VIdx &i0 = fv[0], &i1 = fv[1], &i2 = fv[2], &i3 = fv[3];
        if (!valid(i0) || !valid(i1) || !valid(i2) || !valid(i3)) return;
        const float *p0 = &v[3 * i0.v], *p1 = &v[3 * i1.v], *p2 = &v[3 * i2.v], *p3 = &v[3 * i3.v];
        const float e02x = p2[0] - p0[0], e02y = p2[1] - p0[1], e02z = p2[2] - p0[2];
        const float e13x = p3[0] - p1[0], e13y = p3[1] - p1[1], e13z = p3[2] - p1[2];
        const float s02 = e02x * e02x + e02y * e02y + e02z * e02z;
        const float s13 = e13x * e13x + e13y * e13y + e13z * e13z;
        if (s02 < s13) {
            out.push_back({i0, i1, i2, mat, smooth});
            out.push_back({i0, i2, i3, mat, smooth});
        } else {
            out.push_back({i0, i1, i3, mat, smooth});
            out.push_back({i1, i2, i3, mat, smooth});
        }
        return;
    }
    // ear clipping in the plane of two axes
    size_t axes[2] = {1, 2};
    for (size_t k = 0; k < n; ++k) {
        const VIdx &a = fv[k % n], &b = fv[(k + 1) % n], &c = fv[(k + 2) % n];
        if (!valid(a) || !valid(b) || !valid(c)) continue;
        const float *p0 = &v[3 * a.v], *p1 = &v[3 * b.v], *p2 = &v[3 * c.v];
        const float e0x = p1[0] - p0[0], e0y = p1[1] - p0[1], e0z = p1[2] - p0[2];
        const float e1x = p2[0] - p1[0], e1y = p2[1] - p1[1], e1z = p2[2] - p1[2];
        const float cx = std::fabs(e0y * e1z - e0z * e1y);
        const float cy = std::fabs(e0z * e1x - e0x * e1z);
        const float cz = std::fabs(e0x * e1y - e0y * e1x);
        const float eps = 1.1920929e-7f;
        if (cx > eps || cy > eps || cz > eps) {
            if (!(cx > cy && cx > cz)) {
                axes[0] = 0;
                if (cz > cx && cz > cy) axes[1] = 1;
            }
            break;
        }
    }
    std::vector<VIdx> rem(fv, fv + n);
    size_t guess = 0, iters = rem.size(), prev_n = rem.size();
    auto coord = [&](const VIdx &x, size_t ax) {
        return (x.v < 0 || (size_t)(x.v * 3 + ax) >= vsize) ? 0.0f : v[x.v * 3 + ax];
    };
    while (rem.size() > 3 && iters > 0) {
        const size_t np = rem.size();
        if (guess >= np) guess -= np;
        if (prev_n != np) {
            prev_n = np;
            iters = np;
        } else {
            --iters;
        }
        VIdx ind[3];
        float vx[3], vy[3];
        for (int k = 0; k < 3; ++k) {
            ind[k] = rem[(guess + k) % np];
            vx[k] = coord(ind[k], axes[0]);
            vy[k] = coord(ind[k], axes[1]);
        }
        const float e0x = vx[1] - vx[0], e0y = vy[1] - vy[0], e1x = vx[2] - vx[1], e1y = vy[2] - vy[1];
        const float cross = e0x * e1y - e0y * e1x;
        const float area = (vx[0] * vy[1] - vy[0] * vx[1]) * 0.5f;
        if (cross * area < 0.0f) {
            guess += 1;
            continue;
        }
        bool overlap = false;
        for (size_t o = 3; o < np; ++o) {
            const size_t idx = (guess + o) % np;
            const VIdx &x = rem[idx];
            if (x.v < 0 || (size_t)(x.v * 3 + axes[0]) >= vsize || (size_t)(x.v * 3 + axes[1]) >= vsize)
                continue;
            if (pnpoly3(vx, vy, v[x.v * 3 + axes[0]], v[x.v * 3 + axes[1]])) {
                overlap = true;
                break;
            }
        }
        if (overlap) {
            guess += 1;
            continue;
        }
        out.push_back({ind[0], ind[1], ind[2], mat, smooth});
        size_t r = (guess + 1) % np;
        while (r + 1 < np) {
            rem[r] = rem[r + 1];
            ++r;
        }
        rem.pop_back();
    }
    if (rem.size() == 3) out.push_back({rem[0], rem[1], rem[2], mat, smooth});
}

struct ObjData {
    std::vector<float> v, vn, vt;
    std::vector<Shape> shapes;
    std::vector<MtlMaterial> mats;
};

// ---------------------------------------------------------------------------
// Parallel parse.  The text is cut into chunks at line ends.  A pre-pass counts
// each chunk's lines and v / vn / vt records, so every chunk knows the counts
// before its first line and resolves relative indices exactly as a sequential
// reader would.  Chunks then parse their numbers and face indices in parallel;
// the state-changing lines (g, o, usemtl, mtllib, s, l, p) are kept, in order,
// as events with the face and vertex counts they occur at.  A sequential pass
// replays the events and faces in file order - shapes, materials, smoothing
// groups, triangulation (which sees only the vertices read so far) - so the
// result does not depend on the thread count.

// Line cursor over [p, e): '\n', '\r\n' or '\r' ends a line; the line is
// copied into a reused buffer so the token readers see a C string.
struct LineRange {
    const char *p, *e;
    bool next(std::string &line) {
        if (p >= e) return false;
        const char *q = p;
        while (q < e && *q != '\n' && *q != '\r') ++q;
        line.assign(p, q);
        if (q < e && *q == '\r' && q + 1 < e && q[1] == '\n') ++q;
        p = q < e ? q + 1 : e;
        return true;
    }
};

enum LineKind { kLineSkip, kLineV, kLineVN, kLineVT, kLineLP, kLineF, kLineUsemtl, kLineMtllib, kLineGO, kLineS,
                kLineOther };

// Classifies a line by its first token (leading spaces and tabs skipped).
LineKind classify(const char *t) {
    if (t[0] == '\0' || t[0] == '#') return kLineSkip;
    if (t[0] == 'v' && is_space(t[1])) return kLineV;
    if (t[0] == 'v' && t[1] == 'n' && is_space(t[2])) return kLineVN;
    if (t[0] == 'v' && t[1] == 't' && is_space(t[2])) return kLineVT;
    if ((t[0] == 'l' || t[0] == 'p') && is_space(t[1])) return kLineLP;
    if (t[0] == 'f' && is_space(t[1])) return kLineF;
    if (!strncmp(t, "usemtl", 6)) return kLineUsemtl;
    if (!strncmp(t, "mtllib", 6) && is_space(t[6])) return kLineMtllib;
    if ((t[0] == 'g' || t[0] == 'o') && is_space(t[1])) return kLineGO;
    if (t[0] == 's' && is_space(t[1])) return kLineS;
    return kLineOther;
}

struct Counts {
    size_t lines = 0, nv = 0, nvn = 0, nvt = 0;
};

struct Event {
    LineKind kind;
    size_t nfaces;  // faces of the chunk before this line
    size_t nv;      // vertices of the file before this line
    std::string text;
};

struct Chunk {
    const char *p = nullptr, *e = nullptr;
    Counts cnt, base;  // this chunk's counts; the counts before it
    std::vector<float> v, vn, vt;
    std::vector<VIdx> idx;          // face corners
    std::vector<size_t> face_end;   // end of each face in idx
    std::vector<Event> events;
    size_t err_line = 0;            // 1-based line of the first bad index, 0 = none
    bool err_face = false;
};

void count_chunk(Chunk &c) {
    LineRange lr{c.p, c.e};
    std::string ln;
    while (lr.next(ln)) {
        ++c.cnt.lines;
        const char *t = ln.c_str();
        t += strspn(t, " \t");
        switch (classify(t)) {
            case kLineV: ++c.cnt.nv; break;
            case kLineVN: ++c.cnt.nvn; break;
            case kLineVT: ++c.cnt.nvt; break;
            default: break;
        }
    }
}

void parse_chunk(Chunk &c) {
    LineRange lr{c.p, c.e};
    std::string ln;
    size_t line_no = c.base.lines;
    c.v.reserve(3 * c.cnt.nv);
    c.vn.reserve(3 * c.cnt.nvn);
    c.vt.reserve(2 * c.cnt.nvt);
    while (lr.next(ln)) {
        ++line_no;
        const char *t = ln.c_str();
        t += strspn(t, " \t");
        const LineKind k = classify(t);
        const int nv = (int)(c.base.nv + c.v.size() / 3), nvn = (int)(c.base.nvn + c.vn.size() / 3),
                  nvt = (int)(c.base.nvt + c.vt.size() / 2);
        switch (k) {
            case kLineSkip:
            case kLineOther:
                break;
            case kLineV: {
                t += 2;
                const float x = read_real(&t), y = read_real(&t), z = read_real(&t);
                c.v.push_back(x);
                c.v.push_back(y);
                c.v.push_back(z);
                break;
            }
            case kLineVN: {
                t += 3;
                const float x = read_real(&t), y = read_real(&t), z = read_real(&t);
                c.vn.push_back(x);
                c.vn.push_back(y);
                c.vn.push_back(z);
                break;
            }
            case kLineVT: {
                t += 3;
                const float x = read_real(&t), y = read_real(&t);
                c.vt.push_back(x);
                c.vt.push_back(y);
                break;
            }
            case kLineLP: {
                const char *u = t + 2;
                while (!is_newline(u[0])) {
                    VIdx vi;
                    if (!parse_triple(&u, nv, nvn, nvt, &vi)) {
                        c.err_line = line_no;
                        return;
                    }
                    u += strspn(u, " \t\r");
                }
                c.events.push_back({k, c.face_end.size(), (size_t)nv, std::string()});
                break;
            }
            case kLineF: {
                t += 2;
                t += strspn(t, " \t");
                while (!is_newline(t[0])) {
                    VIdx vi;
                    if (!parse_triple(&t, nv, nvn, nvt, &vi)) {
                        c.err_line = line_no;
                        c.err_face = true;
                        return;
                    }
                    c.idx.push_back(vi);
                    t += strspn(t, " \t\r");
                }
                c.face_end.push_back(c.idx.size());
                break;
            }
            default:
                c.events.push_back({k, c.face_end.size(), (size_t)nv, std::string(t)});
                break;
        }
    }
}

// Runs f(i) for i in [0, n) on up to `threads` threads.
template <class F>
void parallel_for(size_t n, int threads, F f) {
    const size_t nt = std::min<size_t>(n, (size_t)std::max(threads, 1));
    if (nt <= 1) {
        for (size_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    for (size_t w = 0; w < nt; ++w)
        pool.emplace_back([&]() {
            for (size_t i; (i = next.fetch_add(1)) < n;) f(i);
        });
    for (std::thread &th : pool) th.join();
}

int resolve_threads(int threads) {
    if (threads > 0) return std::min(threads, 256);
    const unsigned hw = std::thread::hardware_concurrency();
    return (int)std::min(std::max(hw, 1u), 64u);
}

kgk_status parse_obj(const std::string &path, ObjData &d, int threads) {
    std::string text;
    if (!read_text(path, text)) return fail(KGK_ERR_IO, "cannot open OBJ file " + path);
    const std::string base = dir_of(path);
    // one chunk per call with one thread; else chunks of at least 256 KB, about four per thread
    const size_t min_chunk = (size_t)256 << 10;
    const size_t want =
        threads == 1 ? 1 : std::max<size_t>(1, std::min<size_t>((size_t)threads * 4, text.size() / min_chunk));
    std::vector<Chunk> chunks;
    const char *p = text.data(), *const e = text.data() + text.size();
    for (size_t k = 1; k <= want && p < e; ++k) {
        const char *q = k == want ? e : std::max<const char *>(p, text.data() + text.size() * k / want);
        while (q < e && *q != '\n' && *q != '\r') ++q;  // move to the end of a line
        if (q < e) {
            if (*q == '\r' && q + 1 < e && q[1] == '\n') ++q;
            ++q;
        }
        Chunk c;
        c.p = p;
        c.e = q;
        chunks.push_back(std::move(c));
        p = q;
    }
    parallel_for(chunks.size(), threads, [&](size_t i) { count_chunk(chunks[i]); });
    Counts run;
    for (Chunk &c : chunks) {
        c.base = run;
        run.lines += c.cnt.lines;
        run.nv += c.cnt.nv;
        run.nvn += c.cnt.nvn;
        run.nvt += c.cnt.nvt;
    }
    parallel_for(chunks.size(), threads, [&](size_t i) { parse_chunk(chunks[i]); });
    for (const Chunk &c : chunks)
        if (c.err_line)
            return fail(KGK_ERR_PARSE, path + ":" + std::to_string(c.err_line) +
                                           (c.err_face ? ": bad face index" : ": bad index"));
    d.v.reserve(3 * run.nv);
    d.vn.reserve(3 * run.nvn);
    d.vt.reserve(2 * run.nvt);
    for (const Chunk &c : chunks) {
        d.v.insert(d.v.end(), c.v.begin(), c.v.end());
        d.vn.insert(d.vn.end(), c.vn.begin(), c.vn.end());
        d.vt.insert(d.vt.end(), c.vt.begin(), c.vt.end());
    }
    // sequential replay in file order
    std::map<std::string, int> mat_by_name;
    std::set<std::string> mtl_files;
    struct FaceRef {
        const VIdx *vi;
        size_t n;
        unsigned smooth;
    };
    std::vector<FaceRef> faces;
    bool other = false;  // lines / points in the current primitive group
    int material = -1;
    unsigned smooth = 0;
    Shape shape;
    auto export_group = [&](size_t nv) {
        if (faces.empty() && !other) return false;
        shape.tris.reserve(shape.tris.size() + faces.size());
        for (const FaceRef &f : faces) triangulate(f.vi, f.n, f.smooth, material, d.v, 3 * nv, shape.tris);
        if (other) shape.other_prims = true;
        return true;
    };
    for (const Chunk &c : chunks) {
        size_t f = 0;
        auto take_faces = [&](size_t upto) {
            for (; f < upto; ++f) {
                const size_t b = f ? c.face_end[f - 1] : 0;
                faces.push_back({c.idx.data() + b, c.face_end[f] - b, smooth});
            }
        };
        for (const Event &ev : c.events) {
            take_faces(ev.nfaces);
            const char *t = ev.text.c_str();
            switch (ev.kind) {
                case kLineLP:
                    other = true;
                    break;
                case kLineUsemtl: {
                    t += 6;
                    const std::string name = read_string(&t);
                    auto it = mat_by_name.find(name);
                    const int id = it != mat_by_name.end() ? it->second : -1;
                    if (id != material) {
                        export_group(ev.nv);
                        faces.clear();
                        material = id;
                    }
                    break;
                }
                case kLineMtllib: {
                    t += 7;
                    // file names separated by spaces ('\' escapes a space)
                    std::vector<std::string> names;
                    std::string cur;
                    for (const char *ch = t; *ch; ++ch) {
                        if (*ch == '\\' && ch[1]) {
                            cur += *++ch;
                        } else if (*ch == ' ') {
                            if (!cur.empty()) names.push_back(cur);
                            cur.clear();
                        } else {
                            cur += *ch;
                        }
                    }
                    if (!cur.empty()) names.push_back(cur);
                    for (const std::string &nm : names) {
                        if (mtl_files.count(nm)) break;
                        std::string mt;
                        if (read_text(base + nm, mt)) {
                            parse_mtl(mt, d.mats, mat_by_name);
                            mtl_files.insert(nm);
                            break;
                        }
                    }
                    break;
                }
                case kLineGO:
                    export_group(ev.nv);
                    if (!shape.tris.empty() || (t[0] == 'o' && shape.other_prims)) d.shapes.push_back(std::move(shape));
                    shape = Shape();
                    faces.clear();
                    other = false;
                    break;
                case kLineS: {
                    t += 2;
                    t += strspn(t, " \t");
                    if (t[0] == '\0') break;
                    if (t[0] == '\r' || t[1] == '\n') break;
                    if (strlen(t) >= 3 && t[0] == 'o' && t[1] == 'f' && t[2] == 'f') {
                        smooth = 0;
                    } else {
                        const int g = atoi(t);
                        smooth = g < 0 ? 0u : (unsigned)g;
                    }
                    break;
                }
                default:
                    break;
            }
        }
        take_faces(c.face_end.size());
    }
    const bool ret = export_group(run.nv);
    if (ret || !shape.tris.empty()) d.shapes.push_back(std::move(shape));
    return KGK_OK;
}

kgk_vec vec3(float x, float y, float z) { return kgk_vec{x, y, z, 0.0f}; }

// Vec normalize (struct_Vec.cuh:40-46): a zero vector becomes (10000, 0, 0).
kgk_vec normalize_ref(kgk_vec b) {
    const float l = sqrtf(b.x * b.x + b.y * b.y + b.z * b.z);
    if (l == 0) return vec3(10000, 0, 0);
    return vec3(b.x / l, b.y / l, b.z / l);
}

kgk_material make_mat(int type, int tex, kgk_vec diffuse, kgk_vec emission, float subsurface, float specular,
                      float specularTint, float metallic, float roughness, float anisotropic, float sheen,
                      float sheenTint, float clearcoat, float clearcoatGloss, float ior, float mu_a, float mu_s,
                      float scatter_g) {
    kgk_material m;
    memset(&m, 0, sizeof m);
    m.MATERIAL_TYPE_ID = type;
    m.TEXTURE_BASECOLOR_ID = tex;
    m.diffuse = diffuse;
    m.emission = emission;
    m.subsurface = subsurface;
    m.metallic = metallic;
    m.specular = specular;
    m.specularTint = specularTint;
    m.roughness = roughness;
    m.anisotropic = anisotropic;
    m.sheen = sheen;
    m.sheenTint = sheenTint;
    m.clearcoat = clearcoat;
    m.cloearcoatGloss = clearcoatGloss;
    m.IOR = ior;
    m.mu_a = mu_a;
    m.mu_s = mu_s;
    m.scatter_g = scatter_g;
    return m;
}

}  // namespace

extern "C" {

kgk_status kgk_load_obj_ex(const char *obj_path, const char *hdr_path, const kgk_load_options *opt,
                           kgk_host_scene *out) {
    KGK_GUARD_BEGIN
    if (!obj_path || !out) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_load_obj: NULL argument");
    memset(out, 0, sizeof *out);
    const int model = opt ? opt->material_model : KGK_MATERIALS_REFERENCE;
    if (model != KGK_MATERIALS_REFERENCE && model != KGK_MATERIALS_PBR)
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_load_obj: unknown material_model");
    const int threads = resolve_threads(opt ? opt->threads : 0);
    ObjData d;
    KGK_TRY(parse_obj(obj_path, d, threads));
    const std::string base = dir_of(obj_path);
    // triangles (IO_load_WavefrontObj.cuh:32-88), converted in parallel
    std::vector<size_t> shape_off(d.shapes.size() + 1, 0);
    for (size_t s = 0; s < d.shapes.size(); ++s) shape_off[s + 1] = shape_off[s] + d.shapes[s].tris.size();
    const size_t n_tris = shape_off.back();
    if (n_tris == 0) return fail(KGK_ERR_PARSE, std::string(obj_path) + ": no triangles");
    kgk_triangle *tri_out = (kgk_triangle *)malloc(n_tris * sizeof(kgk_triangle));
    if (!tri_out) return fail(KGK_ERR_OUT_OF_MEMORY, "kgk_load_obj: out of host memory");
    const size_t nv = d.v.size() / 3, nvn = d.vn.size() / 3, nvt = d.vt.size() / 2;
    const size_t block = 1 << 16;
    const size_t n_blocks = (n_tris + block - 1) / block;
    // first bad index per block (triangle index, kind): the earliest is reported
    std::vector<std::pair<size_t, int>> bad(n_blocks, {SIZE_MAX, 0});
    parallel_for(n_blocks, threads, [&](size_t blk) {
        const size_t i0 = blk * block, i1 = std::min(n_tris, i0 + block);
        size_t s = std::upper_bound(shape_off.begin(), shape_off.end(), i0) - shape_off.begin() - 1;
        for (size_t i = i0; i < i1; ++i) {
            while (i >= shape_off[s + 1]) ++s;
            const Tri &tr = d.shapes[s].tris[i - shape_off[s]];
            const VIdx *ix[3] = {&tr.a, &tr.b, &tr.c};
            kgk_vec p[3], n[3], uv[3];
            bool all_n = true;
            for (int k = 0; k < 3; ++k) {
                if (ix[k]->v < 0 || (size_t)ix[k]->v >= nv) {
                    bad[blk] = {i, 0};
                    return;
                }
                p[k] = vec3(d.v[3 * ix[k]->v], d.v[3 * ix[k]->v + 1], d.v[3 * ix[k]->v + 2]);
                // a normal or texcoord index past the file's records counts as
                // absent (tinyobjloader keeps it; load_object would read past
                // its arrays)
                if (ix[k]->vn >= 0 && (size_t)ix[k]->vn < nvn) {
                    n[k] = vec3(d.vn[3 * ix[k]->vn], d.vn[3 * ix[k]->vn + 1], d.vn[3 * ix[k]->vn + 2]);
                } else {
                    all_n = false;
                }
                if (ix[k]->vt >= 0 && (size_t)ix[k]->vt < nvt) {
                    uv[k] = vec3(d.vt[2 * ix[k]->vt], d.vt[2 * ix[k]->vt + 1], 0.0f);
                } else {
                    uv[k] = vec3(0, 0, 0);
                }
            }
            if (!all_n) {
                const kgk_vec e1 = vec3(p[1].x - p[0].x, p[1].y - p[0].y, p[1].z - p[0].z);
                const kgk_vec e2 = vec3(p[2].x - p[0].x, p[2].y - p[0].y, p[2].z - p[0].z);
                const kgk_vec c = vec3(e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x);
                n[0] = n[1] = n[2] = c;
            }
            kgk_triangle &t = tri_out[i];
            memset(&t, 0, sizeof t);
            t.v0 = p[0];
            t.v1 = p[1];
            t.v2 = p[2];
            t.v0_vn = normalize_ref(n[0]);
            t.v1_vn = normalize_ref(n[1]);
            t.v2_vn = normalize_ref(n[2]);
            t.v0_vt = uv[0];
            t.v1_vt = uv[1];
            t.v2_vt = uv[2];
            t.material_id = tr.mat + 1;
            t.is_SmoothNormal = tr.smooth != 0;
            t.shape_id = (int32_t)s;
        }
    });
    for (const auto &b : bad) {
        if (b.first == SIZE_MAX) continue;
        free(tri_out);
        return fail(KGK_ERR_PARSE, std::string(obj_path) + ": vertex index out of range");
    }
    d.shapes.clear();
    d.shapes.shrink_to_fit();
    // materials (scene.cuh:14-18, IO_load_WavefrontObj.cuh:90-124)
    std::vector<kgk_material> mats;
    mats.push_back(make_mat(0, -1, vec3(0.75f, 0.75f, 0.75f), vec3(0, 0, 0), 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f,
                            0.0f, 0.0f, 0.0f, 1.45f, 0.01f, 0.01f, 0.5f));
    std::map<std::string, int> tex_id;
    std::vector<std::string> tex_names;
    for (const MtlMaterial &m : d.mats) {
        kgk_vec diffuse = vec3(m.diffuse[0], m.diffuse[1], m.diffuse[2]);
        const kgk_vec emission = vec3(m.emission[0], m.emission[1], m.emission[2]);
        if (diffuse.x == 0 || diffuse.y == 0 || diffuse.z == 0)
            diffuse = vec3(diffuse.x + 1e-4f, diffuse.y + 1e-4f, diffuse.z + 1e-4f);
        const float spec = sqrtf(m.specular[0] * m.specular[0] + m.specular[1] * m.specular[1] +
                                 m.specular[2] * m.specular[2]);
        int tex = -1;
        if (!m.diffuse_tex.empty()) {
            const size_t k = m.diffuse_tex.find_last_of("/\\");
            const std::string name = k == std::string::npos ? m.diffuse_tex : m.diffuse_tex.substr(k + 1);
            if (!tex_id.count(name)) {
                tex_id[name] = (int)tex_id.size();
                tex_names.push_back(name);
            }
            tex = tex_id[name];
        }
        if (model == KGK_MATERIALS_PBR && m.has_pbr) {
            // Disney from the MTL PBR extension: Pr roughness, Pm metallic,
            // Ps sheen, Pc clearcoat, Pcr clearcoat roughness (gloss = 1 - Pcr),
            // aniso; specular from Ni as F0 / 0.08 (F0 = ((Ni-1)/(Ni+1))^2),
            // 0.5 (F0 = 4 %) without Ni
            auto clamp01 = [](float x) { return std::min(std::max(x, 0.0f), 1.0f); };
            float specular = 0.5f;
            if (m.has_ni && m.ior > 0.0f) {
                const float f0 = ((m.ior - 1.0f) / (m.ior + 1.0f)) * ((m.ior - 1.0f) / (m.ior + 1.0f));
                specular = clamp01(f0 / 0.08f);
            }
            mats.push_back(make_mat(1, tex, diffuse, emission, 0.0f, specular, 0.0f, clamp01(m.metallic),
                                    clamp01(m.roughness), clamp01(m.anisotropy), clamp01(m.sheen), 0.0f,
                                    clamp01(m.clearcoat), 1.0f - clamp01(m.clearcoat_roughness),
                                    m.has_ni ? m.ior : 1.45f, 0.0f, 0.0f, 0.5f));
        } else if (tex >= 0) {
            mats.push_back(make_mat(0, tex, diffuse, emission, 0.0f, spec, 0.0f, m.metallic, m.roughness, 0.0f, 0.0f,
                                    0.0f, 0.0f, 0.0f, m.ior, 0.0f, 0.0f, 0.5f));
        } else {
            mats.push_back(make_mat(0, -1, diffuse, emission, 0.0f, spec, 0.0f, m.metallic, m.roughness, 0.0f, 0.0f,
                                    0.0f, 1.0f, 0.0f, m.ior, 0.01f, 0.01f, 0.0f));
        }
    }
    for (size_t i = 0; i < n_tris; ++i)
        if (tri_out[i].material_id < 0 || (size_t)tri_out[i].material_id >= mats.size()) {
            free(tri_out);
            return fail(KGK_ERR_PARSE, std::string(obj_path) + ": material id out of range");
        }
    // textures (IO_load_images.cuh:9-15: every value + 1e-4), decoded in parallel
    std::vector<kgk_texture> texs(tex_names.size());
    std::vector<kgk_status> tex_st(tex_names.size(), KGK_OK);
    std::vector<std::string> tex_err(tex_names.size());
    parallel_for(tex_names.size(), threads, [&](size_t i) {
        tex_st[i] = load_image_float((base + tex_names[i]).c_str(), &texs[i]);
        if (tex_st[i] != KGK_OK) {
            tex_err[i] = kgk::last_error_message();
            return;
        }
        const size_t cnt = (size_t)texs[i].width * texs[i].height * texs[i].bpp;
        for (size_t k = 0; k < cnt; ++k) texs[i].pixels[k] = (float)((double)texs[i].pixels[k] + 1e-4);
    });
    auto free_all = [&]() {
        for (kgk_texture &x : texs) free(x.pixels);
        free(tri_out);
    };
    for (size_t i = 0; i < tex_names.size(); ++i)
        if (tex_st[i] != KGK_OK) {
            free_all();
            return fail(tex_st[i], tex_err[i]);
        }
    kgk_texture hdr{nullptr, 0, 0, 0};
    if (hdr_path && hdr_path[0]) {
        const kgk_status st = load_image_float(hdr_path, &hdr);
        if (st != KGK_OK) {
            free_all();
            return st;
        }
    }
    out->materials = (kgk_material *)malloc(mats.size() * sizeof(kgk_material));
    out->textures = texs.empty() ? nullptr : (kgk_texture *)malloc(texs.size() * sizeof(kgk_texture));
    if (!out->materials || (!texs.empty() && !out->textures)) {
        free(out->materials);
        free(out->textures);
        free_all();
        free(hdr.pixels);
        memset(out, 0, sizeof *out);
        return fail(KGK_ERR_OUT_OF_MEMORY, "kgk_load_obj: out of host memory");
    }
    out->triangles = tri_out;
    memcpy(out->materials, mats.data(), mats.size() * sizeof(kgk_material));
    if (!texs.empty()) memcpy(out->textures, texs.data(), texs.size() * sizeof(kgk_texture));
    out->n_triangles = n_tris;
    out->n_materials = mats.size();
    out->n_textures = texs.size();
    out->hdr = hdr;
    return KGK_OK;
    KGK_GUARD_END
}

kgk_status kgk_load_obj(const char *obj_path, const char *hdr_path, kgk_host_scene *out) {
    return kgk_load_obj_ex(obj_path, hdr_path, nullptr, out);
}

void kgk_host_scene_free(kgk_host_scene *s) {
    if (!s) return;
    for (size_t i = 0; i < s->n_textures; ++i) free(s->textures[i].pixels);
    free(s->textures);
    free(s->triangles);
    free(s->materials);
    free(s->hdr.pixels);
    memset(s, 0, sizeof *s);
}

kgk_status kgk_scene_load_obj_ex(const char *obj_path, const char *hdr_path, const kgk_load_options *opt,
                                 kgk_scene **out) {
    if (!obj_path || !out) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_load_obj: NULL argument");
    kgk_host_scene hs;
    KGK_TRY(kgk_load_obj_ex(obj_path, hdr_path, opt, &hs));
    const kgk_status st = kgk_scene_create(hs.triangles, hs.n_triangles, hs.materials, hs.n_materials, hs.textures,
                                           hs.n_textures, hs.hdr.pixels ? &hs.hdr : nullptr, out);
    kgk_host_scene_free(&hs);
    return st;
}

kgk_status kgk_scene_load_obj(const char *obj_path, const char *hdr_path, kgk_scene **out) {
    return kgk_scene_load_obj_ex(obj_path, hdr_path, nullptr, out);
}

}  // extern "C"
