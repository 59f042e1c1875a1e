// capi.cpp - the extern "C" entry points of include/kagayaki.h (host C++23).
// Validates arguments, stages host buffers through device memory, and never
// lets an exception or exit() cross the boundary.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "kgk_internal.h"
#include "kgk_scene.h"

namespace kgk {

static thread_local std::string g_last_error;
static thread_local int g_device = 0;

void set_error(const std::string &msg) { g_last_error = msg; }
const std::string &last_error_message() { return g_last_error; }
kgk_status fail(kgk_status st, const std::string &msg) {
    g_last_error = msg;
    return st;
}
kgk_status cuda_fail(cudaError_t e, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return e == cudaErrorMemoryAllocation ? KGK_ERR_OUT_OF_MEMORY : KGK_ERR_CUDA;
}
kgk_status dmalloc(void **p, size_t bytes, const char *what) {
    *p = nullptr;
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        g_last_error = std::string("cudaMalloc(") + std::to_string(bytes) + " B) for " + what + ": " +
                       cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? KGK_ERR_OUT_OF_MEMORY : KGK_ERR_CUDA;
    }
    return KGK_OK;
}
void dfree(void *p) {
    if (p) cudaFree(p);
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

kgk_status check_device() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(KGK_ERR_NO_DEVICE, "no CUDA device is visible");
    }
    if (g_device < 0 || g_device >= n) return fail(KGK_ERR_NO_DEVICE, "device index out of range");
    cudaDeviceProp p;
    KGK_CUDA(cudaGetDeviceProperties(&p, g_device));
    if (p.major != 10 || p.minor != 3)
        return fail(KGK_ERR_NO_DEVICE, "this library is built for sm_103a (GB300); device " +
                                           std::to_string(g_device) + " is sm_" + std::to_string(p.major) +
                                           std::to_string(p.minor));
    KGK_CUDA(cudaSetDevice(g_device));
    return KGK_OK;
}

kgk_status Staging::reserve(size_t bytes) {
    if (bytes <= cap) return KGK_OK;
    dfree(ptr);
    ptr = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 4 + 256;
    KGK_TRY(dmalloc(&ptr, want, "staging buffer"));
    cap = want;
    return KGK_OK;
}

Staging::~Staging() { dfree(ptr); }

}  // namespace kgk

using namespace kgk;

extern "C" {

const char *kgk_version(void) { return "kagayaki-gb300 0.1.0 (sm_103a)"; }

const char *kgk_status_string(kgk_status s) {
    switch (s) {
    case KGK_OK: return "KGK_OK";
    case KGK_ERR_INVALID_ARGUMENT: return "KGK_ERR_INVALID_ARGUMENT";
    case KGK_ERR_OUT_OF_MEMORY: return "KGK_ERR_OUT_OF_MEMORY";
    case KGK_ERR_CUDA: return "KGK_ERR_CUDA";
    case KGK_ERR_NO_DEVICE: return "KGK_ERR_NO_DEVICE";
    case KGK_ERR_IO: return "KGK_ERR_IO";
    case KGK_ERR_PARSE: return "KGK_ERR_PARSE";
    case KGK_ERR_NOT_BUILT: return "KGK_ERR_NOT_BUILT";
    case KGK_ERR_DEVICE_CHECK: return "KGK_ERR_DEVICE_CHECK";
    case KGK_ERR_UNSUPPORTED: return "KGK_ERR_UNSUPPORTED";
    }
    return "KGK_ERR_UNKNOWN";
}

kgk_status kgk_last_error(char *buf, size_t len) {
    if (!buf || len == 0) return KGK_ERR_INVALID_ARGUMENT;
    size_t n = std::min(len - 1, g_last_error.size());
    memcpy(buf, g_last_error.data(), n);
    buf[n] = 0;
    return KGK_OK;
}

kgk_status kgk_set_device(int device) {
    if (device < 0) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_set_device: negative index");
    g_device = device;
    return KGK_OK;
}

kgk_status kgk_scene_create(const kgk_triangle *tris, size_t n_tris, const kgk_material *mats, size_t n_mats,
                            const kgk_texture *textures, size_t n_textures, const kgk_texture *hdr,
                            kgk_scene **out) {
    KGK_GUARD_BEGIN
    if (!out) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_create: out == NULL");
    *out = nullptr;
    if (!tris || n_tris == 0) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_create: no triangles");
    if (!mats || n_mats == 0) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_create: no materials");
    KGK_TRY(check_device());
    auto *s = new kgk_scene();
    s->device = g_device;
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return cuda_fail(e, "cudaStreamCreate");
    }
    kgk_status st = scene_upload(s->dev, tris, n_tris, mats, n_mats, textures, n_textures, hdr, s->stream);
    if (st != KGK_OK) {
        std::string msg = g_last_error;
        kgk_scene_destroy(s);
        g_last_error = msg;
        return st;
    }
    *out = s;
    return KGK_OK;
    KGK_GUARD_END
}

kgk_status kgk_scene_set_textures_rgba8(kgk_scene *s, const kgk_texture_rgba8 *textures, size_t n) {
    if (!s) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_set_textures_rgba8: scene == NULL");
    KGK_CUDA(cudaSetDevice(s->device));
    return scene_set_textures_rgba8(s->dev, textures, n, s->stream);
}

void kgk_scene_destroy(kgk_scene *s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    output_state_free(s);
    render_state_free(s);
    svgf_state_free(s);
    nrc_state_free(s);
    scene_free(s->dev);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

kgk_status kgk_build_bvh(kgk_scene *s, kgk_bvh_info *info) {
    KGK_GUARD_BEGIN
    if (!s) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_build_bvh: scene == NULL");
    KGK_CUDA(cudaSetDevice(s->device));
    BvhBuildStats bs;
    KGK_TRY(bvh_build(s->dev, s->stream, &bs));
    s->built = true;
    if (info) {
        memset(info, 0, sizeof *info);
        info->n_triangles = (uint64_t)s->dev.n_tris;
        info->n_wide_nodes = bs.n_wide;
        info->n_binary_nodes = bs.n_binary;
        info->max_depth = bs.max_depth;
        info->max_leaf_size = bs.max_leaf;
        info->sah_cost = bs.sah;
        info->ms_build = bs.ms;
        info->device_bytes = (uint64_t)s->dev.n_nodes * sizeof(WideNode) + (uint64_t)s->dev.n_tris * 48;
    }
    return KGK_OK;
    KGK_GUARD_END
}

kgk_status kgk_bvh_validate(kgk_scene *s) {
    KGK_GUARD_BEGIN
    if (!s) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_bvh_validate: scene == NULL");
    if (!s->built) return fail(KGK_ERR_NOT_BUILT, "kgk_bvh_validate: call kgk_build_bvh first");
    KGK_CUDA(cudaSetDevice(s->device));
    return bvh_validate(s->dev, s->stream);
    KGK_GUARD_END
}

static kgk_status trace_common(kgk_scene *s, const kgk_ray *rays, const float *tmax, size_t n, int32_t *ids,
                               float *ts, uint8_t *occ, kgk_stats *stats, bool any) {
    if (!s) return fail(KGK_ERR_INVALID_ARGUMENT, "trace: scene == NULL");
    if (!s->built) return fail(KGK_ERR_NOT_BUILT, "trace: call kgk_build_bvh first");
    if (n > 0 && !rays) return fail(KGK_ERR_INVALID_ARGUMENT, "trace: rays == NULL");
    if (!any && n > 0 && (!ids || !ts)) return fail(KGK_ERR_INVALID_ARGUMENT, "trace: face_id/t == NULL");
    if (any && n > 0 && !occ) return fail(KGK_ERR_INVALID_ARGUMENT, "trace: occluded == NULL");
    if (n > 0x7fffffff) return fail(KGK_ERR_INVALID_ARGUMENT, "trace: more than 2^31-1 rays");
    KGK_CUDA(cudaSetDevice(s->device));
    if (stats) memset(stats, 0, sizeof *stats);
    if (n == 0) return KGK_OK;
    const bool rd = is_device_ptr(rays);
    const bool td = tmax ? is_device_ptr(tmax) : true;
    const bool od = any ? is_device_ptr(occ) : (is_device_ptr(ids) && is_device_ptr(ts));
    // staging layout: rays | tmax | ids | t | occ | counters
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += (bytes + 255) & ~size_t(255);
        return o;
    };
    size_t o_rays = rd ? 0 : take(n * sizeof(kgk_ray));
    size_t o_tmax = (tmax && !td) ? take(n * sizeof(float)) : 0;
    size_t o_ids = (!any && !od) ? take(n * sizeof(int32_t)) : 0;
    size_t o_t = (!any && !od) ? take(n * sizeof(float)) : 0;
    size_t o_occ = (any && !od) ? take(n) : 0;
    size_t o_ctr = take(sizeof(TraceCounters));
    KGK_TRY(s->staging.reserve(off));
    char *base = (char *)s->staging.ptr;
    const kgk_ray *d_rays = rd ? rays : (const kgk_ray *)(base + o_rays);
    const float *d_tmax = tmax ? (td ? tmax : (const float *)(base + o_tmax)) : nullptr;
    int32_t *d_ids = (!any) ? (od ? ids : (int32_t *)(base + o_ids)) : nullptr;
    float *d_t = (!any) ? (od ? ts : (float *)(base + o_t)) : nullptr;
    uint8_t *d_occ = any ? (od ? occ : (uint8_t *)(base + o_occ)) : nullptr;
    TraceCounters *d_ctr = (TraceCounters *)(base + o_ctr);
    cudaStream_t st = s->stream;
    if (!rd) KGK_CUDA(cudaMemcpyAsync((void *)d_rays, rays, n * sizeof(kgk_ray), cudaMemcpyHostToDevice, st));
    if (tmax && !td) KGK_CUDA(cudaMemcpyAsync((void *)d_tmax, tmax, n * sizeof(float), cudaMemcpyHostToDevice, st));
    KGK_CUDA(cudaMemsetAsync(d_ctr, 0, sizeof(TraceCounters), st));
    cudaEvent_t e0, e1;
    KGK_CUDA(cudaEventCreate(&e0));
    KGK_CUDA(cudaEventCreate(&e1));
    KGK_CUDA(cudaEventRecord(e0, st));
    kgk_status r = any ? trace_any_dev(s->dev, d_rays, d_tmax, n, d_occ, d_ctr, st)
                       : trace_closest_dev(s->dev, d_rays, n, d_ids, d_t, stats != nullptr, d_ctr, st);
    KGK_CUDA(cudaEventRecord(e1, st));
    if (r != KGK_OK) return r;
    if (!any && !od) {
        KGK_CUDA(cudaMemcpyAsync(ids, d_ids, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        KGK_CUDA(cudaMemcpyAsync(ts, d_t, n * sizeof(float), cudaMemcpyDeviceToHost, st));
    }
    if (any && !od) KGK_CUDA(cudaMemcpyAsync(occ, d_occ, n, cudaMemcpyDeviceToHost, st));
    TraceCounters hc{};
    KGK_CUDA(cudaMemcpyAsync(&hc, d_ctr, sizeof hc, cudaMemcpyDeviceToHost, st));
    KGK_CUDA(cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (stats) {
        if (any) stats->rays_shadow = hc.rays;
        else stats->rays_closest = hc.rays;
        stats->traversal_overflows = hc.overflows;
        stats->nodes_visited = hc.nodes;
        stats->tris_tested = hc.tris;
        stats->ms_device = ms;
    }
    if (hc.overflows)
        return fail(KGK_ERR_DEVICE_CHECK, "trace: " + std::to_string(hc.overflows) +
                                              " rays overflowed the traversal stack");
    return KGK_OK;
}

kgk_status kgk_trace_closest(kgk_scene *s, const kgk_ray *rays, size_t n, int32_t *face_id, float *t,
                             kgk_stats *stats) {
    KGK_GUARD_BEGIN
    return trace_common(s, rays, nullptr, n, face_id, t, nullptr, stats, false);
    KGK_GUARD_END
}

kgk_status kgk_trace_any(kgk_scene *s, const kgk_ray *rays, const float *t_max, size_t n, uint8_t *occluded,
                         kgk_stats *stats) {
    KGK_GUARD_BEGIN
    return trace_common(s, rays, t_max, n, nullptr, nullptr, occluded, stats, true);
    KGK_GUARD_END
}

// Camera_SetUpCamera (struct_Camera.cuh:27-35) and rotate (matrix.cuh:27-38):
// X, then Y, then Z rotation of (0,1,0) and (0,0,-1) in float arithmetic.
static kgk_vec cam_rotate(float x, float y, float z, kgk_vec init) {
    const float rx[4][4] = {{1, 0, 0, 0}, {0, cosf(x), -sinf(x), 0}, {0, sinf(x), cosf(x), 0}, {0, 0, 0, 1}};
    const float ry[4][4] = {{cosf(y), 0, sinf(y), 0}, {0, 1, 0, 0}, {-sinf(y), 0, cosf(y), 0}, {0, 0, 0, 1}};
    const float rz[4][4] = {{cosf(z), -sinf(z), 0, 0}, {sinf(z), cosf(z), 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    float v[4] = {init.x, init.y, init.z, 1.0f}, t[4];
    const float (*ms[3])[4] = {rx, ry, rz};
    for (int m = 0; m < 3; ++m) {
        for (int i = 0; i < 4; ++i) {
            float acc = 0.0f;
            for (int l = 0; l < 4; ++l) acc += ms[m][i][l] * v[l];
            t[i] = acc;
        }
        memcpy(v, t, sizeof v);
    }
    float len = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (len == 0.0f) return {10000.0f, 0.0f, 0.0f, 0.0f};
    return {v[0] / len, v[1] / len, v[2] / len, 0.0f};
}

kgk_status kgk_camera_setup(kgk_vec origin, float dist, float rxd, float ryd, float rzd, int32_t image_height,
                            kgk_camera *out) {
    if (!out) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_camera_setup: out == NULL");
    if (image_height <= 0) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_camera_setup: image_height <= 0");
    const float D2R = 0.01745329f;
    const kgk_vec up = cam_rotate(D2R * rxd, D2R * ryd, D2R * rzd, {0.0f, 1.0f, 0.0f, 0.0f});
    const kgk_vec dir = cam_rotate(D2R * rxd, D2R * ryd, D2R * rzd, {0.0f, 0.0f, -1.0f, 0.0f});
    memset(out, 0, sizeof *out);
    out->CamOrg = {origin.x, origin.y, origin.z, 0.0f};
    out->CamDir = dir;
    out->CamToScreenDist = dist;
    out->ScreenXDir = {dir.y * up.z - dir.z * up.y, dir.z * up.x - dir.x * up.z, dir.x * up.y - dir.y * up.x, 0.0f};
    out->ScreenYDir = up;
    out->PixelSize = 36.0f / (float)image_height;
    return KGK_OK;
}

}  // extern "C"
