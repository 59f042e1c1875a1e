// kgk_internal.h - internal data layout shared by the CUDA translation units
// and the host C++ glue.  Not part of the ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/kagayaki.h"

static_assert(sizeof(kgk_vec) == 16, "Vec must be 16 B (struct_Vec.cuh:4-8)");
static_assert(sizeof(kgk_triangle) == 156, "Triangle must be 156 B (struct_Triangle.cuh:8-20)");
static_assert(offsetof(kgk_triangle, material_id) == 144, "Triangle.material_id offset");
static_assert(offsetof(kgk_triangle, is_SmoothNormal) == 148, "Triangle.is_SmoothNormal offset");
static_assert(offsetof(kgk_triangle, shape_id) == 152, "Triangle.shape_id offset");
static_assert(sizeof(kgk_material) == 96, "Material must be 96 B (struct_Material.cuh:6-11)");
static_assert(offsetof(kgk_material, emission) == 24, "Material.emission offset");
static_assert(offsetof(kgk_material, roughness) == 56, "Material.roughness offset");
static_assert(sizeof(kgk_camera) == 72, "Camera must be 72 B (struct_Camera.cuh:12-18)");
static_assert(offsetof(kgk_camera, ScreenXDir) == 36, "Camera.ScreenXDir offset");
static_assert(offsetof(kgk_camera, PixelSize) == 68, "Camera.PixelSize offset");
static_assert(sizeof(kgk_texture) == 24, "Texture must be 24 B (struct_Texture.cuh:6-8)");
static_assert(sizeof(kgk_ray) == 40, "Ray must be 40 B (struct_Ray.cuh:12-15)");

namespace kgk {

// Smallest float t that the reference accepts: struct_Triangle.cuh:57 rejects
// `t < 1e-5` with 1e-5 a double, i.e. every float below 1e-5 (double).
constexpr float kTMin = 0x1.4f8b5ap-17f;  // 1.000000066e-05
constexpr float kBigT = 1e38f;  // bINF, global_values.cuh:10

// ---------------------------------------------------------------------------
// Compressed 8-wide BVH node (80 B = 5 x 16 B, read as five float4):
//   n0 = (p.x, p.y, p.z, e_x | e_y << 8 | e_z << 16 | imask << 24)
//   n1 = (child_base, tri_base, meta[0..3], meta[4..7])
//   n2 = (qlo_x[0..3], qlo_x[4..7], qhi_x[0..3], qhi_x[4..7])
//   n3 = same for y, n4 = same for z
// Child box a-extent = p.a + q * 2^(e_a - 127).  meta per slot: 0 = empty;
// inner child = 0x20 | (24 + slot) (inner children are stored contiguously
// from child_base in slot order); leaf child = (unary triangle count 1..3) << 5
// | offset of its first triangle from tri_base.
// ---------------------------------------------------------------------------
struct __align__(16) WideNode {
    float4 n0, n1, n2, n3, n4;
};
static_assert(sizeof(WideNode) == 80, "WideNode");

// Binary node of the binned-SAH build (temporary).  lo.w / hi.w carry ints:
// inner: lo.w = left child, hi.w = right child; leaf: lo.w = first ref,
// hi.w = -(count).  cnt = primitives below the node.
struct __align__(16) BinNode {
    float4 lo, hi;
};

struct TexDesc {
    int64_t offset;  // float textures: floats into tex_pixels; RGBA8: texels into tex_rgba8
    int32_t w, h, bpp, rgba8;
};

// Device-resident scene.
struct DevScene {
    int32_t n_tris = 0;
    int32_t n_mats = 0;
    // BVH-order triangle records: 3 float4 per triangle,
    // (v0.xyz, original id as int bits), (v1.xyz, 0), (v2.xyz, 0).
    float4 *tri_rec = nullptr;
    // Input-order vertices (3 float4 per triangle) and shading attributes
    // (4 float4): (n0.xyz, uv0.x) (n1.xyz, uv0.y) (n2.xyz, uv1.x)
    // (uv1.y, uv2.x, uv2.y, bits: material | smooth << 31).
    float4 *verts = nullptr;
    float4 *attr = nullptr;
    kgk_material *mats = nullptr;
    // Textures: float pixels (reference layout) or RGBA8 texels decoded
    // through tex_lut (256 entries: (v/255)^2.2 + 1e-4, the reference loader's
    // value for an 8-bit channel).
    float *tex_pixels = nullptr;
    uchar4 *tex_rgba8 = nullptr;
    float *tex_lut = nullptr;
    TexDesc *tex = nullptr;
    int32_t n_tex = 0;
    int32_t tex_filter = 0;  // per render call: 0 nearest (Texture::get_Color), 1 bilinear
    // Environment (nullptr: none -> background (1,1,1)).
    float *env = nullptr;
    int32_t env_w = 0, env_h = 0, env_bpp = 0;
    float *env_cdf_ref = nullptr;    // reference running FP32 sum over w*h texels
    float2 *env_alias = nullptr;     // unbiased: alias table over w*h texels (threshold, alias index bits)
    float *env_prob = nullptr;       // unbiased: probability of each texel
    float env_total = 0.0f;          // sum of the unbiased weights
    // Face lights.
    float *light_cdf_ref = nullptr;  // reference running FP32 sum over all triangles
    int32_t no_light = 1;
    int32_t *emit_ids = nullptr;     // unbiased: emissive triangles
    float *emit_cdf = nullptr;       // unbiased: normalised CDF over emit_ids (n+1)
    int32_t n_emit = 0;
    float emit_total = 0.0f;         // sum of area * |emission| (double-summed)
    // Bounding box of all vertices (normalises radiance-cache positions).
    float lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    // BVH.
    WideNode *nodes = nullptr;
    int32_t n_nodes = 0;
    int32_t root = 0;
};

// ---------------------------------------------------------------------------
// Error handling inside the library: every failure records a message.
// ---------------------------------------------------------------------------
void set_error(const std::string &msg);
const std::string &last_error_message();  // this thread's last error
kgk_status fail(kgk_status st, const std::string &msg);
kgk_status cuda_fail(cudaError_t e, const char *what);

#define KGK_CUDA(call)                                                       \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) return ::kgk::cuda_fail(e_, #call);           \
    } while (0)

#define KGK_TRY(expr)                                                        \
    do {                                                                     \
        kgk_status s_ = (expr);                                              \
        if (s_ != KGK_OK) return s_;                                         \
    } while (0)

// Device allocation helper (records the failure).
kgk_status dmalloc(void **p, size_t bytes, const char *what);
template <class T> kgk_status dalloc(T **p, size_t count, const char *what) {
    return dmalloc(reinterpret_cast<void **>(p), count * sizeof(T), what);
}
void dfree(void *p);

// ---------------------------------------------------------------------------
// Entry points implemented in the CUDA translation units.
// ---------------------------------------------------------------------------
struct BvhBuildStats {
    uint64_t n_binary = 0, n_wide = 0;
    uint32_t max_depth = 0, max_leaf = 0;
    double sah = 0, ms = 0;
};

kgk_status scene_set_textures_rgba8(DevScene &s, const kgk_texture_rgba8 *tex, size_t n, cudaStream_t st);
kgk_status scene_upload(DevScene &s, const kgk_triangle *tris, size_t n, const kgk_material *mats,
                        size_t nm, const kgk_texture *tex, size_t ntex, const kgk_texture *hdr,
                        cudaStream_t st);
void scene_free(DevScene &s);
kgk_status bvh_build(DevScene &s, cudaStream_t st, BvhBuildStats *out);
kgk_status bvh_validate(const DevScene &s, cudaStream_t st);

// C-ABI entry points: no C++ exception crosses the boundary; a host
// exception (allocation failure) becomes a status.
#define KGK_GUARD_BEGIN try {
#define KGK_GUARD_END                                                        \
    }                                                                        \
    catch (const std::exception &ex) {                                       \
        return fail(KGK_ERR_OUT_OF_MEMORY, std::string("host exception: ") + ex.what()); \
    }                                                                        \
    catch (...) {                                                            \
        return fail(KGK_ERR_OUT_OF_MEMORY, "unknown host exception");      \
    }

struct TraceCounters {
    unsigned long long rays, overflows, nodes, tris;
    unsigned long long fetch;  // next ray to hand out (persistent kernels)
};
kgk_status trace_closest_dev(const DevScene &s, const kgk_ray *rays, size_t n, int32_t *id,
                             float *t, bool count, TraceCounters *ctr_dev, cudaStream_t st);
kgk_status trace_any_dev(const DevScene &s, const kgk_ray *rays, const float *tmax, size_t n,
                         uint8_t *occ, TraceCounters *ctr_dev, cudaStream_t st);

}  // namespace kgk
