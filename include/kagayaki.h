/*
 * kagayaki.h - C ABI of the GB300 render path (sm_103a).
 *
 * A drop-in for the render path of the kagayaki CUDA path tracer: scene
 * upload, BVH build, closest-hit traversal, the path-traced frame, the SVGF
 * denoiser, the learned radiance cache and PNG output.  Every entry point is
 * plain C: pointers and sizes, no C++ or torch types, no exceptions and no
 * exit() across the boundary.  Each returns a kgk_status; kgk_last_error()
 * gives the message of the last failure on the calling thread.
 *
 * Buffer convention: every array argument may be a host pointer or a device
 * pointer (cudaMalloc / managed).  The library inspects the pointer and stages
 * host buffers through its own device memory.  The caller owns its buffers;
 * the library owns all device memory it allocates until kgk_scene_destroy().
 * A scene handle is single-threaded and uses one CUDA stream of its own.
 *
 * Reference citations (file:line) are paths inside RunningOutRate/kagayaki.
 */
#ifndef KAGAYAKI_H_
#define KAGAYAKI_H_

#include <stddef.h>
#include <stdint.h>
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KGK_ABI_VERSION 1

typedef enum kgk_status {
    KGK_OK = 0,
    KGK_ERR_INVALID_ARGUMENT = 1, /* null pointer, size out of range, bad enum   */
    KGK_ERR_OUT_OF_MEMORY = 2,    /* device or host allocation failed            */
    KGK_ERR_CUDA = 3,             /* a CUDA runtime call failed                  */
    KGK_ERR_NO_DEVICE = 4,        /* no CUDA device, or not an sm_103 part       */
    KGK_ERR_IO = 5,               /* file could not be opened / written          */
    KGK_ERR_PARSE = 6,            /* malformed OBJ / MTL / image                 */
    KGK_ERR_NOT_BUILT = 7,        /* trace/render before kgk_build_bvh()         */
    KGK_ERR_DEVICE_CHECK = 8,     /* a kernel's own bounds/iteration check fired */
    KGK_ERR_UNSUPPORTED = 9
} kgk_status;

/* ------------------------------------------------------------------------- */
/* Scene structs, byte-compatible with the reference (sizes and offsets are    */
/* static_asserted below and in the library).                                  */
/* ------------------------------------------------------------------------- */

/* struct_Vec.cuh:4-8 `Vec` (x, y, z + pad), 16 B. */
typedef struct kgk_vec {
    float x, y, z, align;
} kgk_vec;

/* struct_Triangle.cuh:8-20 `Triangle`, 156 B.  vn = per-vertex normals,
 * vt = per-vertex texture coordinates (x = u, y = v). */
typedef struct kgk_triangle {
    kgk_vec v0, v1, v2;
    kgk_vec v0_vn, v1_vn, v2_vn;
    kgk_vec v0_vt, v1_vt, v2_vt;
    int32_t material_id;
    bool is_SmoothNormal;
    int32_t shape_id;
} kgk_triangle;

/* struct_Material.cuh:6-11 `Material`, 96 B.  MATERIAL_TYPE_ID 0 = Lambert,
 * 1 = Disney BRDF; TEXTURE_BASECOLOR_ID -1 = none.  The field name
 * `cloearcoatGloss` keeps the reference's spelling. */
typedef struct kgk_material {
    int32_t MATERIAL_TYPE_ID;
    int32_t TEXTURE_BASECOLOR_ID;
    kgk_vec diffuse, emission;
    float subsurface, metallic, specular, specularTint, roughness, anisotropic,
          sheen, sheenTint, clearcoat, cloearcoatGloss, IOR, mu_a, mu_s, scatter_g;
} kgk_material;

/* struct_Texture.cuh:6-8 `Texture`, 24 B: float pixels, bpp channels. */
typedef struct kgk_texture {
    float *pixels;
    int32_t width, height, bpp;
} kgk_texture;

/* struct_Camera.cuh:12-18 `Camera`, 72 B. */
typedef struct kgk_camera {
    kgk_vec CamOrg;
    kgk_vec CamDir;
    float CamToScreenDist;
    kgk_vec ScreenXDir;
    kgk_vec ScreenYDir;
    float PixelSize;
} kgk_camera;

/* struct_Ray.cuh:12-15 `Ray`, 40 B (dir first, then org). */
typedef struct kgk_ray {
    kgk_vec dir;
    kgk_vec org;
    double _dummy;
} kgk_ray;

typedef struct kgk_scene kgk_scene; /* opaque */

/* ------------------------------------------------------------------------- */
/* Render configuration (replaces the compile-time constants of                */
/* global_values.cuh:17-24, RayTrace.cuh:95 and SVGF.cuh).                     */
/* ------------------------------------------------------------------------- */

typedef enum kgk_estimator {
    /* The reference's estimator, quirks included (radiance starts at 1e-4,
     * un-weighted environment on miss, emission only at depth 0 and on
     * Russian-roulette termination, pixel-corner environment samples, xorshift
     * seeding of render.cuh:29).  Used for image parity with the reference. */
    KGK_ESTIMATOR_COMPAT = 0,
    /* Unbiased path tracing with NEE + MIS (balance heuristic over BSDF, face
     * light and environment sampling), pixel jitter, max-depth cap. */
    KGK_ESTIMATOR_UNBIASED = 1
} kgk_estimator;

typedef struct kgk_render_config {
    int32_t width, height;   /* image size (global_values.cuh:17-18)              */
    int32_t spp;             /* samples per pixel in this call                    */
    int32_t max_depth;       /* max path vertices; <= 0 = unlimited (compat)      */
    int32_t rr_start_depth;  /* Russian roulette may kill from this depth on (3)  */
    int32_t estimator;       /* kgk_estimator                                     */
    uint64_t seed;           /* stream seed (unbiased); ignored by compat         */
    int32_t frame_index;     /* frame number, decorrelates frames                 */
    int32_t accumulate;      /* 1: add this call's samples into the scene's FP64
                                accumulator (converged references)              */
    int32_t wave_paths;      /* paths in flight per wave; 0 = automatic            */
    int32_t count_work;      /* 1: count BVH nodes visited / triangles tested      */
    int32_t write_gbuffer;   /* 1: write the SVGF G-buffer from primary hits       */
    int32_t use_cache;       /* 1: terminate paths into the radiance cache         */
    int32_t profile_stages;  /* 1: time each pipeline stage with CUDA events (the
                              * shadow passes overlap the next bounce's extend);
                              * 2: the same with the stages one after another, so
                              * each stage time is that stage's alone             */
    int32_t texture_filter;  /* 0: nearest (Texture::get_Color, struct_Texture.cuh:
                                12-18); 1: bilinear with wrap-around addressing  */
    int32_t reserved[4];
} kgk_render_config;

/* Work counters of one call.  Rays follow the reference's counting rule: one
 * ray per traversal call (closest, shadow, MIS, reprojection). */
typedef struct kgk_stats {
    uint64_t rays_closest;        /* primary + extension rays                    */
    uint64_t rays_shadow;         /* shadow / occlusion rays                     */
    uint64_t traversal_overflows; /* rays whose traversal stack overflowed      */
    uint64_t nodes_visited;       /* wide nodes intersected by the wavefront's closest-hit
                                     rays (count_work only; not the tail kernel's) */
    uint64_t tris_tested;         /* triangles tested, likewise                 */
    uint64_t paths;               /* camera paths traced                         */
    double ms_device;             /* device time of the call (CUDA events)       */
    uint64_t kernel_launches;     /* kernels this call launched                  */
    double ms_extend;             /* closest-hit stage device time (profile_stages) */
    double ms_shade;              /* shading stage device time (profile_stages)  */
    double ms_shadow;             /* shadow-ray stage device time (profile_stages) */
    uint64_t extend_launches;     /* closest-hit (extend) kernel launches        */
    double ms_tail;               /* tail-kernel device time (profile_stages)    */
    uint64_t rays_tail;           /* closest-hit rays traced by the tail kernel (part of rays_closest) */
} kgk_stats;

typedef struct kgk_bvh_info {
    uint64_t n_triangles;
    uint64_t n_wide_nodes;        /* 8-wide compressed nodes                     */
    uint64_t n_binary_nodes;      /* nodes of the binned-SAH binary tree         */
    uint32_t max_depth;           /* of the wide tree                            */
    uint32_t max_leaf_size;
    double sah_cost;              /* SAH cost of the binary tree                 */
    double ms_build;              /* device time of the build                    */
    uint64_t device_bytes;        /* wide nodes + triangle records               */
} kgk_bvh_info;

/* ------------------------------------------------------------------------- */
/* Library                                                                     */
/* ------------------------------------------------------------------------- */

/* Version string of the library. */
const char *kgk_version(void);
/* Human-readable name of a status code. */
const char *kgk_status_string(kgk_status status);
/* Copies the message of the calling thread's last failure into buf. */
kgk_status kgk_last_error(char *buf, size_t len);
/* Selects the CUDA device for handles created afterwards on this thread. */
kgk_status kgk_set_device(int device);

/* ------------------------------------------------------------------------- */
/* Scene (replaces render_prepare.cuh:33-51, main.cu:110-175 and the device    */
/* symbols ObjectsNum / Light_strength_sum_size / Exists_NoLight / NoHDR set   */
/* through cudaGetSymbolAddress at main.cu:154-175)                             */
/* ------------------------------------------------------------------------- */

/* Uploads triangles, materials, textures (host float pixels) and an optional
 * HDR environment (hdr may be NULL: the reference's HOST_Exists_NoHDR case,
 * background = (1,1,1)).  Also builds the face-light CDF
 * (NextEventEstimation_FaceLight.cuh:8-21) and the environment CDF
 * (ImageBasedLighting.cuh:59-73).  n_tris >= 1, n_mats >= 1. */
kgk_status kgk_scene_create(const kgk_triangle *tris, size_t n_tris,
                            const kgk_material *mats, size_t n_mats,
                            const kgk_texture *textures, size_t n_textures,
                            const kgk_texture *hdr, kgk_scene **out);

/* A scene read from files, in host memory (malloc'ed by the library; free it
 * with kgk_host_scene_free).  hdr.pixels == NULL: no environment. */
typedef struct kgk_host_scene {
    kgk_triangle *triangles;
    size_t n_triangles;
    kgk_material *materials;   /* [0] = the reserved grey material (scene.cuh:14-18) */
    size_t n_materials;
    kgk_texture *textures;     /* float pixels, + 1e-4 as the reference loads them */
    size_t n_textures;
    kgk_texture hdr;
} kgk_host_scene;

/* Reads a Wavefront OBJ with its MTL files and diffuse textures, and an
 * optional environment image (hdr_path may be NULL), into host arrays: the
 * semantics of load_object (FileIO/IO_load_WavefrontObj.cuh:10-127, which
 * parses with tinyobjloader v2.0.0rc10) and load_Textures / load_HDR
 * (FileIO/IO_load_images.cuh:9-29).  MTL files and textures are looked up in
 * the OBJ file's directory.  Vertices without vn (or whose vn index is past
 * the file's normals) take the face normal and without vt (0,0,0), where the
 * reference would read past its arrays.
 * Images: every format stbi_loadf reads: PNG, JPEG (baseline and progressive),
 * BMP, TGA, GIF (first frame), PSD, Softimage PIC, binary PNM and Radiance
 * .hdr. */
kgk_status kgk_load_obj(const char *obj_path, const char *hdr_path, kgk_host_scene *out);
void kgk_host_scene_free(kgk_host_scene *scene);

/* Loading options (no counterpart in the reference, whose load_object has
 * none).  material_model: KGK_MATERIALS_REFERENCE converts every MTL material
 * as load_object does (Lambert, IO_load_WavefrontObj.cuh:90-124);
 * KGK_MATERIALS_PBR makes a material that has any key of the MTL PBR
 * extension (Pr, Pm, Ps, Pc, Pcr, aniso) a Disney material: roughness Pr,
 * metallic Pm, sheen Ps, clearcoat Pc, clearcoat gloss 1 - Pcr, anisotropic
 * aniso (each clamped to [0,1]), base colour Kd / map_Kd, emission Ke,
 * specular ((Ni-1)/(Ni+1))^2 / 0.08 clamped (0.5 without Ni); the others stay
 * as the reference converts them.  threads: parse and conversion threads
 * (0 = all hardware threads, at most 64); the result is the same for every
 * thread count.  A NULL options pointer means all zeros. */
typedef enum kgk_material_model {
    KGK_MATERIALS_REFERENCE = 0,
    KGK_MATERIALS_PBR = 1
} kgk_material_model;

typedef struct kgk_load_options {
    int32_t material_model;
    int32_t threads;
    int32_t reserved[6];
} kgk_load_options;

kgk_status kgk_load_obj_ex(const char *obj_path, const char *hdr_path, const kgk_load_options *options,
                           kgk_host_scene *out);

/* stbi_loadf (FileIO/IO_load_images.cuh:10): the image as float pixels with
 * its own channel count; 8-bit colour channels (v/255)^2.2, alpha v/255, .hdr
 * as stored.  Free with kgk_image_free. */
kgk_status kgk_load_image(const char *path, kgk_texture *out);
void kgk_image_free(kgk_texture *image);

/* kgk_load_obj followed by kgk_scene_create (render_prepare's load_object +
 * load_HDR, render_prepare.cuh:35-37). */
kgk_status kgk_scene_load_obj(const char *obj_path, const char *hdr_path, kgk_scene **out);
kgk_status kgk_scene_load_obj_ex(const char *obj_path, const char *hdr_path, const kgk_load_options *options,
                                 kgk_scene **out);

/* An 8-bit RGBA texture, 4 bytes per texel, rows from the top.  Kept as bytes
 * on the device (a quarter of the float texture's memory); a colour channel v
 * reads as (v/255)^2.2 + 1e-4, the value the reference's loader
 * (stbi_loadf + load_image, FileIO/IO_load_images.cuh:9-15) gives the same
 * 8-bit file, so nearest-filtered renders equal those of the float texture. */
typedef struct kgk_texture_rgba8 {
    const uint8_t *pixels;
    int32_t width, height;
} kgk_texture_rgba8;

/* Replaces the scene's textures with n RGBA8 textures (materials'
 * TEXTURE_BASECOLOR_ID index them; n must cover every id in use). */
kgk_status kgk_scene_set_textures_rgba8(kgk_scene *scene, const kgk_texture_rgba8 *textures, size_t n);

void kgk_scene_destroy(kgk_scene *scene);

/* Builds the acceleration structure on the GPU: binned SAH into a binary tree,
 * collapsed into 8-wide compressed nodes.  Replaces construct_BVH
 * (ConstructBVH.cuh:204) and MallocAndSetBVHtreeOnDevice
 * (struct_BVH_node.cuh:72-83).  info may be NULL. */
kgk_status kgk_build_bvh(kgk_scene *scene, kgk_bvh_info *info);

/* Structural check of the built BVH on the host (every triangle referenced
 * once, child boxes enclose their contents).  Returns KGK_ERR_DEVICE_CHECK and
 * a message when an invariant fails. */
kgk_status kgk_bvh_validate(kgk_scene *scene);

/* ------------------------------------------------------------------------- */
/* Traversal (replaces willIntersectWithTriangle_nonRecursive,                 */
/* ConstructBVH.cuh:286-368)                                                   */
/* ------------------------------------------------------------------------- */

/* Closest hit of n rays: face_id[i] = index of the hit triangle in the scene's
 * input order or -1 on a miss, t[i] = hit distance (1e38 on a miss).  A hit
 * needs t >= 1e-5 (struct_Triangle.cuh:57); equal distances resolve to the
 * smaller face id.  Intersection is watertight FP32. */
kgk_status kgk_trace_closest(kgk_scene *scene, const kgk_ray *rays, size_t n,
                             int32_t *face_id, float *t, kgk_stats *stats);

/* Occlusion of n rays: occluded[i] = 1 when any triangle is hit with
 * 1e-5 <= t < t_max[i] (t_max may be NULL: unbounded). */
kgk_status kgk_trace_any(kgk_scene *scene, const kgk_ray *rays, const float *t_max,
                         size_t n, uint8_t *occluded, kgk_stats *stats);

/* ------------------------------------------------------------------------- */
/* Camera and frame                                                            */
/* ------------------------------------------------------------------------- */

/* Camera_SetUpCamera (struct_Camera.cuh:27-35): Euler rotation in degrees
 * (X then Y then Z), PixelSize = 36 / image_height. */
kgk_status kgk_camera_setup(kgk_vec origin, float cam_to_screen_dist, float rotate_x_deg,
                            float rotate_y_deg, float rotate_z_deg, int32_t image_height,
                            kgk_camera *out);

/* Renders one frame: spp paths per pixel, out[y*width+x] = mean radiance of
 * this call's samples (x,y,z; align = 1).  Replaces render<<<>>>
 * (render.cuh:21-49, main.cu:199) with a wavefront pipeline.  prev_cam may be
 * NULL (no reprojection).  When cfg->accumulate is set, the samples are also
 * added to the scene's FP64 accumulator (see kgk_accum_*).  out may be host
 * or device memory, or NULL: the frame then stays on the device, in the
 * scene, for kgk_svgf_output(noisy = NULL) (no counterpart in the reference). */
kgk_status kgk_render(kgk_scene *scene, const kgk_camera *cam, const kgk_camera *prev_cam,
                      const kgk_render_config *cfg, kgk_vec *out, kgk_stats *stats);

/* FP64 accumulator of kgk_render(accumulate=1): resets it for width x height. */
kgk_status kgk_accum_reset(kgk_scene *scene, int32_t width, int32_t height);
/* Reads the accumulator: mean[p] (x,y,z) and, when var != NULL, the per-pixel
 * sample variance of the mean, both in FP64.  n_samples may be NULL. */
kgk_status kgk_accum_read(kgk_scene *scene, double *mean_rgb, double *var_rgb,
                          uint64_t *n_samples);

/* ------------------------------------------------------------------------- */
/* SVGF (replaces ApplySVGF, SVGF.cuh:495-522)                                  */
/* ------------------------------------------------------------------------- */

typedef enum kgk_svgf_mode {
    /* The reference's filter in its race-free reading: temporal accumulation,
     * moments, 3x3 variance blur and 5x5 a-trous passes with full-image
     * barriers between phases, the reference's constants and quirks. */
    KGK_SVGF_COMPAT = 0,
    /* Standard SVGF: working reprojection from the previous camera, temporal
     * alpha, n a-trous iterations with edge-stopping sigmas. */
    KGK_SVGF_STANDARD = 1,
    /* Temporal reuse alone: the standard filter's reprojection and history
     * (alpha) with no spatial pass - for frames that are already smooth, such
     * as those the radiance cache terminates into.  A sample whose
     * demodulated luminance exceeds 4x the brightest of its eight neighbours
     * (1e-3 added) is scaled down to that bound before it enters the
     * history, and the reprojected history is clamped, per channel, to the
     * range of the current 3x3 neighbourhood (pixels that hit). */
    KGK_SVGF_TEMPORAL = 2
} kgk_svgf_mode;

typedef struct kgk_svgf_config {
    int32_t mode;            /* kgk_svgf_mode                                   */
    int32_t width, height;
    int32_t frame_index;     /* 0 resets history (SVGF.cuh:502-504)            */
    int32_t atrous_iterations;   /* 5                                          */
    int32_t atrous_repeats;      /* compat: 5 (the k-loop of SVGF.cuh:486)     */
    float alpha;             /* temporal blend of the new frame (0.2)          */
    float sigma_z, sigma_n, sigma_l; /* 1, 128, 4                              */
    int32_t reserved[6];
} kgk_svgf_config;

/* Filters the frame last rendered with write_gbuffer=1 (its G-buffer, and
 * for KGK_SVGF_STANDARD the camera it was rendered with).  noisy is read and
 * filtered is written (both width*height kgk_vec, host or device).  The
 * filter keeps its history in the scene handle. */
kgk_status kgk_svgf(kgk_scene *scene, const kgk_svgf_config *cfg, const kgk_vec *noisy,
                    kgk_vec *filtered);

/* kgk_svgf for a frame loop (no counterpart in the reference, whose main.cu
 * filters, then gamma-converts and writes PNGs on the host, IO_save_png.cuh).
 *   noisy    NULL = the frame the last kgk_render kept on the device (out = NULL)
 *   filtered NULL = not written (else host or device, as kgk_svgf)
 *   rgba8    NULL = not written; else width*height*4 bytes (host or device):
 *            the filtered frame with save_png's tone mapping (powf(x, 1/2.2f),
 *            clamp, x255 truncated, alpha 255; bytes equal to
 *            kgk_tonemap_rgba8's), written in the filter's last pass
 *   async    0 = return when every output is written.  1 = return once the
 *            work is queued: a host rgba8 buffer is filled by a copy on a
 *            second stream that overlaps the scene's next calls, and is
 *            complete when kgk_scene_sync returns; the buffer must stay valid
 *            until then.  The copy overlaps only when rgba8 is pinned memory
 *            (kgk_host_alloc, or cudaHostAlloc / cudaHostRegister); pageable
 *            memory is copied before the call returns.  A host `filtered`
 *            buffer makes the call wait.
 * At least one of filtered and rgba8 must be given. */
kgk_status kgk_svgf_output(kgk_scene *scene, const kgk_svgf_config *cfg, const kgk_vec *noisy,
                           kgk_vec *filtered, uint8_t *rgba8, int32_t async);
/* Waits for the scene's queued work and output copies. */
kgk_status kgk_scene_sync(kgk_scene *scene);
/* Page-locked host memory for overlapped output copies; free with kgk_host_free. */
kgk_status kgk_host_alloc(size_t bytes, void **out);
void kgk_host_free(void *ptr);

/* struct_SVGFBuffers.cuh:7-23 `SVGFBuffer`, 112 B: the reference's per-pixel
 * G-buffer and filter state. */
typedef struct kgk_svgf_buffer {
    kgk_vec Albedo, Emission, Normal, ColorHistory;
    int32_t ObjectID, MaterialID;
    int32_t PosLastFrameI[2];
    float PosLastFrameF[2];
    int32_t sampleNum;
    float MomentOne, MomentTwo, Variance, Depth;
    bool willApplyATrousFilter, willApplyTemporalAccumulation;
} kgk_svgf_buffer;

/* ApplySVGF (SVGF.cuh:495-522) over the reference's own buffers, in its
 * race-free reading (a full-image barrier at every __syncthreads): result is
 * read and rewritten (ColorHistory at the end, SVGF.cuh:492), filtered
 * receives the output image, cur is updated like the reference updates it,
 * prev is read (and initialised when frame == 0).  All arrays hold
 * width*height records, host or device.  Uses the current device and its own
 * stream; synchronous. */
kgk_status kgk_svgf_apply(kgk_vec *result, kgk_vec *filtered, kgk_svgf_buffer *prev,
                          kgk_svgf_buffer *cur, int32_t width, int32_t height, int32_t frame);

/* evaluate_Disney_BRDF and evaluate_Disney_BRDF_pdf (Disney_BRDF.cuh:118-183)
 * on the device, as the compat estimator evaluates them, with the parameters
 * RayTrace derives from the material (RayTrace.cuh:85-92): for n direction
 * triples (3 floats each) wo (toward the light), wi (toward the viewer) and
 * the normal, brdf receives 3 floats and pdf 1 float per triple.  Buffers
 * may be host or device memory; uses the current device; synchronous. */
kgk_status kgk_disney_eval(const kgk_material *material, int32_t n, const float *wo, const float *wi,
                           const float *normal, float *brdf, float *pdf);

/* The reference-layout G-buffer of the frame last rendered with
 * write_gbuffer = 1: the SVGFBuffer records the reference's render() fills
 * for its caller (every record initialised as render.cuh:28 does, then at the
 * primary hit Albedo after texture mapping, Emission, the normal facing the
 * ray, ObjectID, MaterialID and Depth as RayTrace.cuh:66-82; ObjectID -1 on
 * a miss; PosLastFrameI/F left at (-1, -1), where struct_Camera.cuh:109-110
 * leaves them).  This is the `cur` argument kgk_svgf_apply takes.
 * out = width*height records, host or device; synchronous. */
kgk_status kgk_gbuffer_records(kgk_scene *scene, kgk_svgf_buffer *out);

/* Largest image (width * height) kgk_svgf_apply_noalloc accepts. */
#define KGK_SVGF_NOALLOC_MAX_PIXELS (512 * 512)

/* kgk_svgf_apply without any device allocation, for callers that cannot call
 * cudaMalloc: applications that hand all device memory to their own pool
 * allocator at start-up, and per-frame loops that must not allocate because
 * cudaMalloc / cudaFree synchronise the whole device.  No counterpart in the
 * reference (its ApplySVGF allocates nothing because its scratch is fixed
 * 1920x1920 globals, SVGF.cuh:109-110).
 *
 * Same filter and results as kgk_svgf_apply.  Differences:
 *  - result, filtered, prev and cur must be device memory (host buffers are
 *    rejected: staging them would allocate);
 *  - width * height <= KGK_SVGF_NOALLOC_MAX_PIXELS, else
 *    KGK_ERR_INVALID_ARGUMENT;
 *  - the work runs on `cuda_stream` (a cudaStream_t, NULL = the default
 *    stream) and the call returns when it has finished;
 *  - scratch comes from one fixed device array of ~34 MB inside the library,
 *    which every GPU that loads the library holds until the process exits.
 *    All calls share it: calls that overlap on the GPU (for instance from two
 *    host threads on two streams) race and give undefined results.  Each call
 *    writes every scratch word it reads, so what an earlier call left there
 *    does not matter.
 * The first call on each device looks the array's device address up
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  The address is kept for the life of the
 * process: after cudaDeviceReset on a device, do not call this function on
 * that device again. */
kgk_status kgk_svgf_apply_noalloc(kgk_vec *result, kgk_vec *filtered, kgk_svgf_buffer *prev,
                                  kgk_svgf_buffer *cur, int32_t width, int32_t height, int32_t frame,
                                  void *cuda_stream);

/* ------------------------------------------------------------------------- */
/* Learned radiance cache (no counterpart in the reference)                    */
/* ------------------------------------------------------------------------- */

/* A small MLP (64 encoded inputs -> 5 hidden layers of 64, ReLU -> RGB) that
 * kgk_render(use_cache=1) queries where a path's spread exceeds the pixel
 * footprint, trained online every frame on the tracer's own radiance samples.
 * BF16 weights and activations on the tensor cores, FP32 accumulation, FP32
 * master weights, Adam, relative-L2 loss with dynamic loss scaling.
 * Raw query = 13 floats: position normalised to the scene box (3), shading
 * normal (3), direction toward the viewer (3), roughness, albedo (3). */
typedef struct kgk_nrc_config {
    int32_t width;              /* hidden width: 64 (0 = 64) or 128              */
    int32_t hidden_layers;      /* 5                                             */
    float learning_rate;        /* Adam, 1e-2                                    */
    int32_t train_paths;        /* training paths per frame, 65,536              */
    int32_t train_suffix_max;   /* bounces a training path runs past its query, 4 */
    int32_t train_steps;        /* Adam steps per frame, 4                       */
    float spread_c;             /* termination: path spread^2 > c * footprint^2  */
    uint64_t seed;              /* weight initialisation                          */
    int32_t reserved[8];
} kgk_nrc_config;

/* (Re)initialises the scene's cache with He-uniform weights. */
kgk_status kgk_nrc_init(kgk_scene *scene, const kgk_nrc_config *cfg);
/* FP32 master weights, layer by layer, each (out, in) row-major: W x 64,
 * 4 x (W x W), then 3 x W for hidden width W (20,672 floats at width 64,
 * 74,112 at width 128). */
kgk_status kgk_nrc_set_weights(kgk_scene *scene, const float *w, size_t n);
kgk_status kgk_nrc_get_weights(kgk_scene *scene, float *w, size_t n);
/* Predictions (n x 3) for n raw queries (n x 13). */
kgk_status kgk_nrc_infer(kgk_scene *scene, const float *raw, size_t n, float *out);
/* Gradient of the mean relative-L2 loss over the batch w.r.t. the weights
 * (as many floats as the weights, loss scale removed) and the loss; weights
 * unchanged.  raw / target: host or device; grad and loss: host memory. */
kgk_status kgk_nrc_gradients(kgk_scene *scene, const float *raw, const float *target, size_t n,
                             float *grad, float *loss);
/* `steps` Adam steps on one batch; loss (host memory, may be NULL) = the
 * last step's loss. */
kgk_status kgk_nrc_train(kgk_scene *scene, const float *raw, const float *target, size_t n,
                         int32_t steps, float *loss);
/* Current dynamic loss scale. */
kgk_status kgk_nrc_loss_scale(kgk_scene *scene, float *scale);

/* ------------------------------------------------------------------------- */
/* Image output (replaces save_png, FileIO/IO_save_png.cuh:34-56)              */
/* ------------------------------------------------------------------------- */

/* gamma 1/2.2, then clamp to [0,1], then x255 truncated, alpha 255
 * (IO_save_png.cuh:26,7,47-52): out = width*height*4 bytes.  A NaN (also from
 * a negative value) gives 0.  A device img is tone-mapped on the device (the
 * same bytes); out may then be host or device memory. */
kgk_status kgk_tonemap_rgba8(const kgk_vec *img, int32_t width, int32_t height, uint8_t *out);
/* Writes the tone-mapped image as an RGBA8 PNG. */
kgk_status kgk_save_png(const kgk_vec *img, int32_t width, int32_t height, const char *path);
/* Writes the image's linear RGB (no tone mapping) as an OpenEXR file: one
 * part, scanlines without compression, channels B, G, R as FP32 (half == 0)
 * or FP16 (half != 0, rounded to nearest even, overflow to infinity).  img
 * may be host or device memory.  No counterpart in the reference. */
kgk_status kgk_save_exr(const kgk_vec *img, int32_t width, int32_t height, int32_t half, const char *path);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* KAGAYAKI_H_ */
