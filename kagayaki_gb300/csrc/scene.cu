// scene.cu - scene upload: triangle/material/texture/environment data into
// the device layout of kgk_internal.h, plus the light and environment CDFs.
//
// Replaces render_prepare (render_prepare.cuh:33-51) and the uploads of
// main.cu:110-175.  The reference-estimator CDFs are the reference's own
// sequential FP32 running sums (NextEventEstimation_FaceLight.cuh:8-21,
// ImageBasedLighting.cuh:59-73) computed on the host in input order; this file
// is compiled with -ffp-contract=off so the sums round the same way on every
// host.  The unbiased estimator gets normalised CDFs accumulated in double.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "kgk_device.cuh"
#include "kgk_internal.h"

namespace kgk {
namespace {

inline float int_bits_as_float(int i) {
    float f;
    memcpy(&f, &i, sizeof f);
    return f;
}

struct HV {
    float x, y, z;
};
inline HV hv(const kgk_vec &v) { return {v.x, v.y, v.z}; }
inline HV sub(HV a, HV b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline HV crs(HV a, HV b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float hlen(HV a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }

// Triangle::area (struct_Triangle.cuh:106-108).
inline float tri_area(const kgk_triangle &t) {
    return 0.5f * hlen(crs(sub(hv(t.v1), hv(t.v0)), sub(hv(t.v2), hv(t.v0))));
}

bool is_device_ptr(const void *p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

template <class T> kgk_status to_host(const T *p, size_t n, std::vector<T> &out) {
    out.resize(n);
    if (is_device_ptr(p)) {
        KGK_CUDA(cudaMemcpy(out.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost));
    } else {
        memcpy(out.data(), p, n * sizeof(T));
    }
    return KGK_OK;
}

template <class T> kgk_status upload(T **dst, const T *src, size_t n, const char *what, cudaStream_t st) {
    KGK_TRY(dalloc(dst, n > 0 ? n : 1, what));
    if (n > 0) KGK_CUDA(cudaMemcpyAsync(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice, st));
    return KGK_OK;
}

// Triangle records (156 B, the reference's layout) to the device layout:
// vertices (3 float4) and attributes (normals, texcoords, material id with
// the smooth-normal flag in bit 31; 4 float4).  A repacking, no arithmetic.
__global__ void k_tri_soa(const kgk_triangle *__restrict__ raw, size_t n, float4 *__restrict__ verts,
                          float4 *__restrict__ attr) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const kgk_triangle &t = raw[i];
        verts[3 * i] = make_float4(t.v0.x, t.v0.y, t.v0.z, 0.0f);
        verts[3 * i + 1] = make_float4(t.v1.x, t.v1.y, t.v1.z, 0.0f);
        verts[3 * i + 2] = make_float4(t.v2.x, t.v2.y, t.v2.z, 0.0f);
        const unsigned char smooth = reinterpret_cast<const unsigned char *>(&t)[148];
        const unsigned bits = ((unsigned)t.material_id & 0x7fffffffu) | (smooth ? 0x80000000u : 0u);
        attr[4 * i] = make_float4(t.v0_vn.x, t.v0_vn.y, t.v0_vn.z, t.v0_vt.x);
        attr[4 * i + 1] = make_float4(t.v1_vn.x, t.v1_vn.y, t.v1_vn.z, t.v0_vt.y);
        attr[4 * i + 2] = make_float4(t.v2_vn.x, t.v2_vn.y, t.v2_vn.z, t.v1_vt.x);
        attr[4 * i + 3] = make_float4(t.v1_vt.y, t.v2_vt.x, t.v2_vt.y, __uint_as_float(bits));
    }
}

// Runs f(begin, end) over [0, n) in blocks on the host's threads.
template <class F>
void host_blocks(size_t n, size_t block, F f) {
    const size_t nb = (n + block - 1) / block;
    const unsigned hw = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    const size_t nt = std::min<size_t>(nb, hw);
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (size_t b; (b = next.fetch_add(1)) < nb;) f(b * block, std::min(n, (b + 1) * block));
    };
    std::vector<std::thread> pool;
    for (size_t k = 1; k < nt; ++k) pool.emplace_back(work);
    work();
    for (std::thread &th : pool) th.join();
}

}  // namespace

kgk_status scene_upload(DevScene &s, const kgk_triangle *tris_in, size_t n, const kgk_material *mats_in,
                        size_t nm, const kgk_texture *tex, size_t ntex, const kgk_texture *hdr,
                        cudaStream_t st) {
    if (!tris_in || n == 0) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_create: no triangles");
    if (!mats_in || nm == 0) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_create: no materials");
    if (n > (size_t)600000000) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_create: too many triangles");
    if (ntex > 0 && !tex) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_create: textures == NULL");
    // Host triangle records are read in place: copied as they are to the
    // device (and repacked there by k_tri_soa) while host threads check the
    // material ids and compute the bounds and the per-triangle light terms.
    std::vector<kgk_triangle> tris_copy;
    const kgk_triangle *tris = tris_in;
    const bool tris_dev = is_device_ptr(tris_in);
    if (tris_dev) {
        KGK_TRY(to_host(tris_in, n, tris_copy));
        tris = tris_copy.data();
    }
    std::vector<kgk_material> mats;
    KGK_TRY(to_host(mats_in, nm, mats));
    for (size_t i = 0; i < nm; ++i)
        if (mats[i].TEXTURE_BASECOLOR_ID >= (int)ntex || mats[i].TEXTURE_BASECOLOR_ID < -1)
            return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_create: material " + std::to_string(i) +
                                                      " names a missing texture");
    struct DevBuf {
        kgk_triangle *p = nullptr;
        ~DevBuf() { dfree(p); }
    } raw;
    KGK_TRY(dalloc(&raw.p, n, "triangle records (upload)"));
    KGK_TRY(dalloc(&s.verts, 3 * n, "triangle vertices"));
    KGK_TRY(dalloc(&s.attr, 4 * n, "triangle attributes"));
    // emission length per material; per-triangle term area * |emission|
    // (calculate_Lss's summand, the same float expression)
    std::vector<float> elen(nm), term(n);
    for (size_t m = 0; m < nm; ++m) elen[m] = hlen(hv(mats[m].emission));
    const size_t block = 1 << 16;
    const size_t nb = (n + block - 1) / block;
    std::vector<size_t> bad(nb, SIZE_MAX);
    std::vector<float> blo(3 * nb, INFINITY), bhi(3 * nb, -INFINITY);
    auto host_pass = [&]() {
    host_blocks(n, block, [&](size_t i0, size_t i1) {
        const size_t b = i0 / block;
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (size_t i = i0; i < i1; ++i) {
            const kgk_triangle &t = tris[i];
            if (t.material_id < 0 || (size_t)t.material_id >= nm) {
                if (bad[b] == SIZE_MAX) bad[b] = i;
                continue;
            }
            const kgk_vec *vs[3] = {&t.v0, &t.v1, &t.v2};
            for (const kgk_vec *v : vs) {
                const float c[3] = {v->x, v->y, v->z};
                for (int a = 0; a < 3; ++a) {
                    lo[a] = std::fmin(lo[a], c[a]);
                    hi[a] = std::fmax(hi[a], c[a]);
                }
            }
            term[i] = tri_area(t) * elen[t.material_id];
        }
        for (int a = 0; a < 3; ++a) {
            blo[3 * b + a] = lo[a];
            bhi[3 * b + a] = hi[a];
        }
    });
    };
    {
        // the host pass runs while this thread copies the records (a copy
        // from pageable memory holds the calling thread until it is staged)
        std::thread pass(host_pass);
        const cudaError_t e1 = cudaMemcpyAsync(raw.p, tris_in, n * sizeof(kgk_triangle),
                                               tris_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st);
        if (e1 == cudaSuccess)
            k_tri_soa<<<(int)std::min<size_t>((n + 255) / 256, 8192), 256, 0, st>>>(raw.p, n, s.verts, s.attr);
        const cudaError_t e2 = cudaGetLastError();
        pass.join();
        if (e1 != cudaSuccess) return cuda_fail(e1, "triangle upload");
        if (e2 != cudaSuccess) return cuda_fail(e2, "k_tri_soa");
    }
    for (size_t b = 0; b < nb; ++b)
        if (bad[b] != SIZE_MAX) {
            cudaStreamSynchronize(st);
            const size_t i = bad[b];
            return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_create: triangle " + std::to_string(i) +
                                                      " has material_id " + std::to_string(tris[i].material_id) +
                                                      " outside [0, " + std::to_string(nm) + ")");
        }
    s.n_tris = (int32_t)n;
    s.n_mats = (int32_t)nm;
    for (int a = 0; a < 3; ++a) {
        s.lo[a] = INFINITY;
        s.hi[a] = -INFINITY;
        for (size_t b = 0; b < nb; ++b) {
            s.lo[a] = std::fmin(s.lo[a], blo[3 * b + a]);
            s.hi[a] = std::fmax(s.hi[a], bhi[3 * b + a]);
        }
    }
    KGK_TRY(upload(&s.mats, mats.data(), nm, "materials", st));
    // face lights: the reference's running FP32 sum (calculate_Lss), in input order
    {
        std::vector<float> cdf(n);
        std::vector<int32_t> ids;
        std::vector<double> w;
        cdf[0] = term[0];
        for (size_t i = 1; i < n; ++i) cdf[i] = cdf[i - 1] + term[i];
        s.no_light = cdf[n - 1] == 0.0f ? 1 : 0;
        KGK_TRY(upload(&s.light_cdf_ref, cdf.data(), n, "light CDF", st));
        double total = 0.0;
        for (size_t i = 0; i < n; ++i) {
            const float e = elen[tris[i].material_id];
            if (!(e > 0.0f)) continue;  // the weight would be 0 (or NaN): not an emitter
            const double wi = (double)tri_area(tris[i]) * (double)e;
            if (wi > 0.0) {
                ids.push_back((int32_t)i);
                w.push_back(wi);
                total += wi;
            }
        }
        s.n_emit = (int32_t)ids.size();
        s.emit_total = (float)total;
        std::vector<float> ecdf(ids.size() + 1);
        double acc = 0.0;
        ecdf[0] = 0.0f;
        for (size_t k = 0; k < ids.size(); ++k) {
            acc += w[k];
            ecdf[k + 1] = (float)(acc / total);
        }
        if (!ids.empty()) ecdf.back() = 1.0f;
        KGK_TRY(upload(&s.emit_ids, ids.data(), ids.size(), "emitter list", st));
        KGK_TRY(upload(&s.emit_cdf, ecdf.data(), ecdf.size(), "emitter CDF", st));
        KGK_CUDA(cudaStreamSynchronize(st));
    }

    // textures
    if (ntex > 0) {
        std::vector<kgk_texture> th;
        KGK_TRY(to_host(tex, ntex, th));
        std::vector<TexDesc> desc(ntex);
        size_t total = 0;
        for (size_t i = 0; i < ntex; ++i) {
            if (!th[i].pixels || th[i].width <= 0 || th[i].height <= 0 || th[i].bpp < 1 || th[i].bpp > 4)
                return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_create: texture " + std::to_string(i) +
                                                          " needs pixels, a size and 1 to 4 channels");
            desc[i].offset = (int64_t)total;
            desc[i].w = th[i].width;
            desc[i].h = th[i].height;
            desc[i].bpp = th[i].bpp;
            total += (size_t)th[i].width * th[i].height * th[i].bpp;
        }
        KGK_TRY(dalloc(&s.tex_pixels, total, "texture pixels"));
        for (size_t i = 0; i < ntex; ++i) {
            size_t cnt = (size_t)th[i].width * th[i].height * th[i].bpp;
            KGK_CUDA(cudaMemcpy(s.tex_pixels + desc[i].offset, th[i].pixels, cnt * sizeof(float),
                                is_device_ptr(th[i].pixels) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
        }
        KGK_TRY(upload(&s.tex, desc.data(), ntex, "texture table", st));
        s.n_tex = (int32_t)ntex;
    }

    // environment
    if (hdr && hdr->pixels) {
        const int w = hdr->width, h = hdr->height, bpp = hdr->bpp;
        if (w <= 0 || h <= 0 || bpp < 3) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_create: bad HDR size");
        const size_t npx = (size_t)w * h;
        std::vector<float> px;
        KGK_TRY(to_host(hdr->pixels, npx * bpp, px));
        KGK_TRY(upload(&s.env, px.data(), px.size(), "environment", st));
        s.env_w = w;
        s.env_h = h;
        s.env_bpp = bpp;
        // reference running sum (calculate_Lss_HDR)
        const float PIH = 3.14159265358979323846263383f;
        std::vector<float> cdf(npx);
        float v = 1.0f;
        cdf[0] = hlen({px[0], px[1], px[2]}) * cosf((v - 0.5f) * PIH);
        for (size_t i = 1; i < npx; ++i) {
            v = 1.0f - (float)(int)(i / (size_t)w) / (float)h;
            cdf[i] = cdf[i - 1] + hlen({px[bpp * i], px[bpp * i + 1], px[bpp * i + 2]}) * cosf((v - 0.5f) * PIH);
        }
        KGK_TRY(upload(&s.env_cdf_ref, cdf.data(), npx, "environment CDF", st));
        // unbiased: texel weight = |rgb| * cos(latitude of the row centre),
        // sampled in O(1) through an alias table (Vose's construction)
        std::vector<double> q(npx);
        double total = 0.0;
        for (int r = 0; r < h; ++r) {
            const double c = cos((0.5 - (r + 0.5) / h) * M_PI);
            for (int x = 0; x < w; ++x) {
                const float *p = &px[((size_t)r * w + x) * bpp];
                const double l = sqrt((double)p[0] * p[0] + (double)p[1] * p[1] + (double)p[2] * p[2]);
                q[(size_t)r * w + x] = l * c + 1e-30;
                total += q[(size_t)r * w + x];
            }
        }
        std::vector<float> prob(npx);
        std::vector<float2> alias(npx);
        std::vector<size_t> small, large;
        for (size_t i = 0; i < npx; ++i) {
            prob[i] = (float)(q[i] / total);
            q[i] = q[i] / total * (double)npx;  // scaled: mean 1
            (q[i] < 1.0 ? small : large).push_back(i);
        }
        while (!small.empty() && !large.empty()) {
            const size_t a = small.back(), l = large.back();
            small.pop_back();
            alias[a] = make_float2((float)q[a], int_bits_as_float((int)l));
            q[l] = (q[l] + q[a]) - 1.0;
            if (q[l] < 1.0) {
                large.pop_back();
                small.push_back(l);
            }
        }
        for (size_t i : large) alias[i] = make_float2(1.0f, int_bits_as_float((int)i));
        for (size_t i : small) alias[i] = make_float2(1.0f, int_bits_as_float((int)i));  // rounding leftovers
        s.env_total = (float)total;
        KGK_TRY(upload(&s.env_alias, alias.data(), alias.size(), "environment alias table", st));
        KGK_TRY(upload(&s.env_prob, prob.data(), prob.size(), "environment texel probabilities", st));
        KGK_CUDA(cudaStreamSynchronize(st));
    }
    return KGK_OK;
}

kgk_status scene_set_textures_rgba8(DevScene &s, const kgk_texture_rgba8 *tex, size_t n, cudaStream_t st) {
    if (n > 0 && !tex) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_set_textures_rgba8: textures == NULL");
    std::vector<TexDesc> desc(n);
    size_t total = 0;
    for (size_t i = 0; i < n; ++i) {
        if (!tex[i].pixels || tex[i].width <= 0 || tex[i].height <= 0)
            return fail(KGK_ERR_INVALID_ARGUMENT,
                        "kgk_scene_set_textures_rgba8: texture " + std::to_string(i) + " needs pixels and a size");
        desc[i].offset = (int64_t)total;
        desc[i].w = tex[i].width;
        desc[i].h = tex[i].height;
        desc[i].bpp = 4;
        desc[i].rgba8 = 1;
        total += (size_t)tex[i].width * tex[i].height;
    }
    // materials may only name textures that exist
    std::vector<kgk_material> mats(s.n_mats);
    KGK_CUDA(cudaMemcpy(mats.data(), s.mats, mats.size() * sizeof(kgk_material), cudaMemcpyDeviceToHost));
    for (const kgk_material &m : mats)
        if (m.TEXTURE_BASECOLOR_ID >= (int)n)
            return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_set_textures_rgba8: a material names texture " +
                                                      std::to_string(m.TEXTURE_BASECOLOR_ID) + " of " +
                                                      std::to_string(n));
    dfree(s.tex_pixels);
    dfree(s.tex_rgba8);
    dfree(s.tex);
    s.tex_pixels = nullptr;
    s.tex_rgba8 = nullptr;
    s.tex = nullptr;
    s.n_tex = 0;
    if (n == 0) return KGK_OK;
    KGK_TRY(dalloc(&s.tex_rgba8, total, "RGBA8 texels"));
    for (size_t i = 0; i < n; ++i) {
        const size_t cnt = (size_t)tex[i].width * tex[i].height;
        KGK_CUDA(cudaMemcpy(s.tex_rgba8 + desc[i].offset, tex[i].pixels, cnt * 4,
                            is_device_ptr(tex[i].pixels) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
    }
    if (!s.tex_lut) {
        float lut[256];
        for (int v = 0; v < 256; ++v) lut[v] = (float)((double)powf(v / 255.0f, 2.2f) + 1e-4);
        KGK_TRY(upload(&s.tex_lut, lut, 256, "texture decode table", st));
    }
    KGK_TRY(upload(&s.tex, desc.data(), n, "texture table", st));
    s.n_tex = (int32_t)n;
    KGK_CUDA(cudaStreamSynchronize(st));
    return KGK_OK;
}

void scene_free(DevScene &s) {
    dfree(s.tri_rec);
    dfree(s.verts);
    dfree(s.attr);
    dfree(s.mats);
    dfree(s.tex_pixels);
    dfree(s.tex_rgba8);
    dfree(s.tex_lut);
    dfree(s.tex);
    dfree(s.env);
    dfree(s.env_cdf_ref);
    dfree(s.env_alias);
    dfree(s.env_prob);
    dfree(s.light_cdf_ref);
    dfree(s.emit_ids);
    dfree(s.emit_cdf);
    dfree(s.nodes);
    s = DevScene();
}

}  // namespace kgk
