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
// Differences by design: vertices without vn take the face's geometric normal
// and without vt take (0, 0, 0) (the reference indexes missing entries); MTL
// files and textures are looked up in the OBJ file's directory (the reference
// uses the working directory); malformed input returns an error instead of
// exiting.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <set>
#include <string>
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

// tinyobjloader's number grammar (see the file comment).
bool parse_double(const char *s, const char *end, double *out) {
    if (s >= end) return false;
    double mant = 0.0;
    int expo = 0;
    char sign = '+', esign = '+';
    const char *c = s;
    int read = 0;
    bool more = false, lead_dot = false;
    if (*c == '+' || *c == '-') {
        sign = *c++;
        if (c != end && *c == '.') lead_dot = true;
    } else if (is_digit(*c)) {
    } else if (*c == '.') {
        lead_dot = true;
    } else {
        return false;
    }
    more = c != end;
    if (!lead_dot) {
        while (more && is_digit(*c)) {
            mant *= 10;
            mant += (int)(*c - '0');
            ++c;
            ++read;
            more = c != end;
        }
        if (read == 0) return false;
    }
    if (!more) goto assemble;
    if (*c == '.') {
        ++c;
        read = 1;
        more = c != end;
        static const double kPow10Neg[8] = {1.0, 0.1, 0.01, 0.001, 0.0001, 0.00001, 0.000001, 0.0000001};
        while (more && is_digit(*c)) {
            mant += (int)(*c - '0') * (read < 8 ? kPow10Neg[read] : std::pow(10.0, -read));
            ++read;
            ++c;
            more = c != end;
        }
    } else if (*c == 'e' || *c == 'E') {
    } else {
        goto assemble;
    }
    if (!more) goto assemble;
    if (*c == 'e' || *c == 'E') {
        ++c;
        more = c != end;
        if (more && (*c == '+' || *c == '-')) {
            esign = *c++;
        } else if (is_digit(*c)) {
        } else {
            return false;
        }
        read = 0;
        more = c != end;
        while (more && is_digit(*c)) {
            if (expo > 2147483647 / 10) return false;
            expo *= 10;
            expo += (int)(*c - '0');
            ++c;
            ++read;
            more = c != end;
        }
        expo *= (esign == '+' ? 1 : -1);
        if (read == 0) return false;
    }
assemble:
    *out = (sign == '+' ? 1 : -1) * (expo ? std::ldexp(mant * std::pow(5.0, expo), expo) : mant);
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

struct Face {
    std::vector<VIdx> vi;
    unsigned smooth = 0;
};
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
        if (t[0] == 'N' && t[1] == 'i' && is_space(t[2])) { t += 2; m.ior = read_real(&t); continue; }
        if (t[0] == 'P' && t[1] == 'r' && is_space(t[2])) { t += 2; m.roughness = read_real(&t); continue; }
        if (t[0] == 'P' && t[1] == 'm' && is_space(t[2])) { t += 2; m.metallic = read_real(&t); continue; }
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

// Emits the triangles of one polygon (tinyobjloader's "simple" triangulation).
void triangulate(const Face &f, int mat, const std::vector<float> &v, std::vector<Tri> &out) {
    const size_t n = f.vi.size();
    if (n < 3) return;
    if (n == 3) {
        out.push_back({f.vi[0], f.vi[1], f.vi[2], mat, f.smooth});
        return;
    }
    auto valid = [&](const VIdx &x) { return x.v >= 0 && (size_t)(3 * x.v + 2) < v.size(); };
    if (n == 4) {
        const VIdx &i0 = f.vi[0], &i1 = f.vi[1], &i2 = f.vi[2], &i3 = f.vi[3];
        if (!valid(i0) || !valid(i1) || !valid(i2) || !valid(i3)) return;
        const float *p0 = &v[3 * i0.v], *p1 = &v[3 * i1.v], *p2 = &v[3 * i2.v], *p3 = &v[3 * i3.v];
        const float e02x = p2[0] - p0[0], e02y = p2[1] - p0[1], e02z = p2[2] - p0[2];
        const float e13x = p3[0] - p1[0], e13y = p3[1] - p1[1], e13z = p3[2] - p1[2];
        const float s02 = e02x * e02x + e02y * e02y + e02z * e02z;
        const float s13 = e13x * e13x + e13y * e13y + e13z * e13z;
        if (s02 < s13) {
            out.push_back({i0, i1, i2, mat, f.smooth});
            out.push_back({i0, i2, i3, mat, f.smooth});
        } else {
            out.push_back({i0, i1, i3, mat, f.smooth});
            out.push_back({i1, i2, i3, mat, f.smooth});
        }
        return;
    }
    // ear clipping in the plane of two axes
    size_t axes[2] = {1, 2};
    for (size_t k = 0; k < n; ++k) {
        const VIdx &a = f.vi[k % n], &b = f.vi[(k + 1) % n], &c = f.vi[(k + 2) % n];
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
    std::vector<VIdx> rem = f.vi;
    size_t guess = 0, iters = rem.size(), prev_n = rem.size();
    auto coord = [&](const VIdx &x, size_t ax) {
        return (x.v < 0 || (size_t)(x.v * 3 + ax) >= v.size()) ? 0.0f : v[x.v * 3 + ax];
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
            if (x.v < 0 || (size_t)(x.v * 3 + axes[0]) >= v.size() || (size_t)(x.v * 3 + axes[1]) >= v.size())
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
        out.push_back({ind[0], ind[1], ind[2], mat, f.smooth});
        size_t r = (guess + 1) % np;
        while (r + 1 < np) {
            rem[r] = rem[r + 1];
            ++r;
        }
        rem.pop_back();
    }
    if (rem.size() == 3) out.push_back({rem[0], rem[1], rem[2], mat, f.smooth});
}

struct ObjData {
    std::vector<float> v, vn, vt;
    std::vector<Shape> shapes;
    std::vector<MtlMaterial> mats;
};

kgk_status parse_obj(const std::string &path, ObjData &d) {
    std::string text;
    if (!read_text(path, text)) return fail(KGK_ERR_IO, "cannot open OBJ file " + path);
    const std::string base = dir_of(path);
    std::map<std::string, int> mat_by_name;
    std::set<std::string> mtl_files;
    std::vector<Face> faces;
    bool other = false;  // lines / points in the current primitive group
    int material = -1;
    unsigned smooth = 0;
    Shape shape;
    auto export_group = [&]() {
        if (faces.empty() && !other) return false;
        for (const Face &f : faces) triangulate(f, material, d.v, shape.tris);
        if (other) shape.other_prims = true;
        return true;
    };
    Lines lines{text};
    std::string ln;
    size_t line_no = 0;
    while (lines.next(ln)) {
        ++line_no;
        if (!ln.empty() && ln.back() == '\n') ln.pop_back();
        if (!ln.empty() && ln.back() == '\r') ln.pop_back();
        if (ln.empty()) continue;
        const char *t = ln.c_str();
        t += strspn(t, " \t");
        if (t[0] == '\0' || t[0] == '#') continue;
        if (t[0] == 'v' && is_space(t[1])) {
            t += 2;
            const float x = read_real(&t), y = read_real(&t), z = read_real(&t);
            d.v.push_back(x);
            d.v.push_back(y);
            d.v.push_back(z);
            continue;
        }
        if (t[0] == 'v' && t[1] == 'n' && is_space(t[2])) {
            t += 3;
            const float x = read_real(&t), y = read_real(&t), z = read_real(&t);
            d.vn.push_back(x);
            d.vn.push_back(y);
            d.vn.push_back(z);
            continue;
        }
        if (t[0] == 'v' && t[1] == 't' && is_space(t[2])) {
            t += 3;
            const float x = read_real(&t), y = read_real(&t);
            d.vt.push_back(x);
            d.vt.push_back(y);
            continue;
        }
        if ((t[0] == 'l' || t[0] == 'p') && is_space(t[1])) {
            t += 2;
            while (!is_newline(t[0])) {
                VIdx vi;
                if (!parse_triple(&t, (int)(d.v.size() / 3), (int)(d.vn.size() / 3), (int)(d.vt.size() / 2), &vi))
                    return fail(KGK_ERR_PARSE, path + ":" + std::to_string(line_no) + ": bad index");
                t += strspn(t, " \t\r");
            }
            other = true;
            continue;
        }
        if (t[0] == 'f' && is_space(t[1])) {
            t += 2;
            t += strspn(t, " \t");
            Face f;
            f.smooth = smooth;
            while (!is_newline(t[0])) {
                VIdx vi;
                if (!parse_triple(&t, (int)(d.v.size() / 3), (int)(d.vn.size() / 3), (int)(d.vt.size() / 2), &vi))
                    return fail(KGK_ERR_PARSE, path + ":" + std::to_string(line_no) + ": bad face index");
                f.vi.push_back(vi);
                t += strspn(t, " \t\r");
            }
            faces.push_back(std::move(f));
            continue;
        }
        if (!strncmp(t, "usemtl", 6)) {
            t += 6;
            const std::string name = read_string(&t);
            auto it = mat_by_name.find(name);
            const int id = it != mat_by_name.end() ? it->second : -1;
            if (id != material) {
                export_group();
                faces.clear();
                material = id;
            }
            continue;
        }
        if (!strncmp(t, "mtllib", 6) && is_space(t[6])) {
            t += 7;
            // file names separated by spaces ('\' escapes a space)
            std::vector<std::string> names;
            std::string cur;
            for (const char *c = t; *c; ++c) {
                if (*c == '\\' && c[1]) {
                    cur += *++c;
                } else if (*c == ' ') {
                    if (!cur.empty()) names.push_back(cur);
                    cur.clear();
                } else {
                    cur += *c;
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
            continue;
        }
        if ((t[0] == 'g' || t[0] == 'o') && is_space(t[1])) {
            export_group();
            if (!shape.tris.empty() || (t[0] == 'o' && shape.other_prims)) d.shapes.push_back(std::move(shape));
            shape = Shape();
            faces.clear();
            other = false;
            continue;
        }
        if (t[0] == 's' && is_space(t[1])) {
            t += 2;
            t += strspn(t, " \t");
            if (t[0] == '\0') continue;
            if (t[0] == '\r' || t[1] == '\n') continue;
            if (strlen(t) >= 3 && t[0] == 'o' && t[1] == 'f' && t[2] == 'f') {
                smooth = 0;
            } else {
                const int g = atoi(t);
                smooth = g < 0 ? 0u : (unsigned)g;
            }
            continue;
        }
    }
    const bool ret = export_group();
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

kgk_status kgk_load_obj(const char *obj_path, const char *hdr_path, kgk_host_scene *out) {
    if (!obj_path || !out) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_load_obj: NULL argument");
    memset(out, 0, sizeof *out);
    ObjData d;
    KGK_TRY(parse_obj(obj_path, d));
    const std::string base = dir_of(obj_path);
    // triangles (IO_load_WavefrontObj.cuh:32-88)
    std::vector<kgk_triangle> tris;
    const size_t nv = d.v.size() / 3, nvn = d.vn.size() / 3, nvt = d.vt.size() / 2;
    for (size_t s = 0; s < d.shapes.size(); ++s) {
        for (const Tri &tr : d.shapes[s].tris) {
            const VIdx *ix[3] = {&tr.a, &tr.b, &tr.c};
            kgk_vec p[3], n[3], uv[3];
            bool all_n = true;
            for (int k = 0; k < 3; ++k) {
                if (ix[k]->v < 0 || (size_t)ix[k]->v >= nv)
                    return fail(KGK_ERR_PARSE, std::string(obj_path) + ": vertex index out of range");
                p[k] = vec3(d.v[3 * ix[k]->v], d.v[3 * ix[k]->v + 1], d.v[3 * ix[k]->v + 2]);
                if (ix[k]->vn >= 0) {
                    if ((size_t)ix[k]->vn >= nvn)
                        return fail(KGK_ERR_PARSE, std::string(obj_path) + ": normal index out of range");
                    n[k] = vec3(d.vn[3 * ix[k]->vn], d.vn[3 * ix[k]->vn + 1], d.vn[3 * ix[k]->vn + 2]);
                } else {
                    all_n = false;
                }
                if (ix[k]->vt >= 0) {
                    if ((size_t)ix[k]->vt >= nvt)
                        return fail(KGK_ERR_PARSE, std::string(obj_path) + ": texcoord index out of range");
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
            kgk_triangle t;
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
            tris.push_back(t);
        }
    }
    if (tris.empty()) return fail(KGK_ERR_PARSE, std::string(obj_path) + ": no triangles");
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
        if (!m.diffuse_tex.empty()) {
            const size_t k = m.diffuse_tex.find_last_of("/\\");
            const std::string name = k == std::string::npos ? m.diffuse_tex : m.diffuse_tex.substr(k + 1);
            if (!tex_id.count(name)) {
                tex_id[name] = (int)tex_id.size();
                tex_names.push_back(name);
            }
            mats.push_back(make_mat(0, tex_id[name], diffuse, emission, 0.0f, spec, 0.0f, m.metallic, m.roughness,
                                    0.0f, 0.0f, 0.0f, 0.0f, 0.0f, m.ior, 0.0f, 0.0f, 0.5f));
        } else {
            mats.push_back(make_mat(0, -1, diffuse, emission, 0.0f, spec, 0.0f, m.metallic, m.roughness, 0.0f, 0.0f,
                                    0.0f, 1.0f, 0.0f, m.ior, 0.01f, 0.01f, 0.0f));
        }
    }
    for (const kgk_triangle &t : tris)
        if (t.material_id < 0 || (size_t)t.material_id >= mats.size())
            return fail(KGK_ERR_PARSE, std::string(obj_path) + ": material id out of range");
    // textures (IO_load_images.cuh:9-15: every value + 1e-4)
    std::vector<kgk_texture> texs(tex_names.size());
    auto free_all = [&]() {
        for (kgk_texture &x : texs) free(x.pixels);
    };
    for (size_t i = 0; i < tex_names.size(); ++i) {
        const kgk_status st = load_image_float((base + tex_names[i]).c_str(), &texs[i]);
        if (st != KGK_OK) {
            free_all();
            return st;
        }
        const size_t cnt = (size_t)texs[i].width * texs[i].height * texs[i].bpp;
        for (size_t k = 0; k < cnt; ++k) texs[i].pixels[k] = (float)((double)texs[i].pixels[k] + 1e-4);
    }
    kgk_texture hdr{nullptr, 0, 0, 0};
    if (hdr_path && hdr_path[0]) {
        const kgk_status st = load_image_float(hdr_path, &hdr);
        if (st != KGK_OK) {
            free_all();
            return st;
        }
    }
    out->triangles = (kgk_triangle *)malloc(tris.size() * sizeof(kgk_triangle));
    out->materials = (kgk_material *)malloc(mats.size() * sizeof(kgk_material));
    out->textures = texs.empty() ? nullptr : (kgk_texture *)malloc(texs.size() * sizeof(kgk_texture));
    if (!out->triangles || !out->materials || (!texs.empty() && !out->textures)) {
        free(out->triangles);
        free(out->materials);
        free(out->textures);
        free_all();
        free(hdr.pixels);
        memset(out, 0, sizeof *out);
        return fail(KGK_ERR_OUT_OF_MEMORY, "kgk_load_obj: out of host memory");
    }
    memcpy(out->triangles, tris.data(), tris.size() * sizeof(kgk_triangle));
    memcpy(out->materials, mats.data(), mats.size() * sizeof(kgk_material));
    if (!texs.empty()) memcpy(out->textures, texs.data(), texs.size() * sizeof(kgk_texture));
    out->n_triangles = tris.size();
    out->n_materials = mats.size();
    out->n_textures = texs.size();
    out->hdr = hdr;
    return KGK_OK;
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

kgk_status kgk_scene_load_obj(const char *obj_path, const char *hdr_path, kgk_scene **out) {
    if (!obj_path || !out) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_load_obj: NULL argument");
    kgk_host_scene hs;
    KGK_TRY(kgk_load_obj(obj_path, hdr_path, &hs));
    const kgk_status st = kgk_scene_create(hs.triangles, hs.n_triangles, hs.materials, hs.n_materials, hs.textures,
                                           hs.n_textures, hs.hdr.pixels ? &hs.hdr : nullptr, out);
    kgk_host_scene_free(&hs);
    return st;
}

}  // extern "C"
