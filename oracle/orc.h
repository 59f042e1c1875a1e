/*
 * orc.h - CPU oracle: a plain-C restatement of the reference's render-path
 * arithmetic.  TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg use it, and only as the checker or the timed
 * CPU baseline; the product never links it.
 *
 * Structs are the reference's layouts (kagayaki.h mirrors them): Triangle
 * 156 B, Material 96 B, Ray 40 B, Camera 72 B, Vec 16 B.
 */
#ifndef KGK_ORC_H_
#define KGK_ORC_H_
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Reference ray/triangle test (struct_Triangle.cuh:30-58): returns 1 and t,
 * u, v when the Cramer-rule barycentrics pass u,v >= 0, u+v <= 1, t >= 1e-5. */
int orc_intersect_ref(const void *tri, const void *ray, float *t, float *u, float *v);

/* Closest hit over all triangles with the reference test; ties resolve to the
 * smaller index (the reference's strict `>` over an index-ordered face list). */
void orc_closest_brute(const void *tris, int64_t n, const void *rays, int64_t nrays,
                       int32_t *face_id, float *t, int nthreads);

/* Per-ray fragility flags of the reference decision: bit 0 = another
 * triangle passes with exactly the same t as the closest; bit 1 = a triangle
 * at or before the closest t has a barycentric (u, v or 1-u-v) within 4 ulp of
 * its edge, or t within 4 ulp of 1e-5.  Rays with flags set may legitimately
 * differ between the reference's Cramer test and a watertight test. */
void orc_classify(const void *tris, int64_t n, const void *rays, int64_t nrays,
                  const int32_t *face_id, const float *t, uint8_t *flags, int nthreads);

/* A CPU BVH (binned SAH, binary) with conservative culling, so that
 * orc_bvh_closest() returns exactly what orc_closest_brute() would. */
typedef struct orc_bvh orc_bvh;
orc_bvh *orc_bvh_build(const void *tris, int64_t n);
void orc_bvh_closest(const orc_bvh *b, const void *rays, int64_t nrays, int32_t *face_id,
                     float *t, int nthreads);
void orc_bvh_free(orc_bvh *b);

/* Reference xorshift (struct_Xorshift.cuh:10-31). */
uint64_t orc_xorshift(uint64_t s);
float orc_random_range(uint64_t *seed, float lo, float hi);

/* Camera_SetUpCamera (struct_Camera.cuh:27-35) with PixelSize = 36/height. */
void orc_camera_setup(const float *org, float dist, float rx, float ry, float rz,
                      int image_height, void *camera_out);

/* gamma 1/2.2 -> clamp [0,1] -> x255 truncate, alpha 255
 * (FileIO/IO_save_png.cuh:26,7,47-52). img: npx Vec (16 B). */
void orc_tonemap_rgba8(const float *img, int64_t npx, uint8_t *out);

/* Face-light CDF (NextEventEstimation_FaceLight.cuh:8-21): running FP32 sum
 * of area * |emission| in input order. */
void orc_light_cdf(const void *tris, int64_t n, const void *mats, float *cdf);
/* Environment CDF (ImageBasedLighting.cuh:59-73). */
void orc_env_cdf(const float *pixels, int w, int h, int bpp, float *cdf);

/* Compat estimator (the reference's RayTrace, RayTrace.cuh:9-109 with its
 * NEE / RR / sampling helpers) for all pixels but 0 of a width x height
 * image, `frames` samples per pixel with the persistent-seed chain of
 * render.cuh:29,42.  out = frames * npx * 3 floats.  textures: n_tex Texture
 * structs (host float pixels).  hdr may be NULL.  Closest hits are the
 * brute-force reference test (small scenes).  The PT-MIS ray of
 * NextEventEstimation_PathTracing.cuh contributes nothing (it returns on a hit
 * and reads face -1 on a miss); it still draws its random numbers.  Returns
 * the number of traversal calls the reference would make. */
int64_t orc_render_compat(const void *tris, int64_t n, const void *mats, int64_t nm,
                          const void *textures, int n_tex, const float *hdr, int hdr_w,
                          int hdr_h, int hdr_bpp, const void *cam, int width, int height,
                          int frames, int nthreads, float *out);

/* evaluate_Disney_BRDF (outgoing = toward the light, incoming = toward the
 * viewer) and evaluate_Disney_BRDF_pdf (Disney_BRDF.cuh:118-183). */
void orc_disney_eval(const void *mat, int n, const float *wo, const float *wi, const float *nrm,
                     float *brdf, float *pdf);
/* The compat estimator over a pixel list with closest hits from a CPU BVH. */
int64_t orc_render_compat_px(const void *tris, int64_t n, const void *mats, const orc_bvh *bvh,
                             const float *hdr, int hdr_w, int hdr_h, int hdr_bpp, const void *cam,
                             int width, int height, const int32_t *px_list, int64_t n_px, int nthreads,
                             float *out);
/* ApplySVGF (SVGF.cuh:495-522) in its race-free reading: every
 * __syncthreads() is a barrier over the whole image.  result, filtered: npx
 * Vec; prev, cur: npx SVGFBuffer records (112 B, struct_SVGFBuffers.cuh). */
void orc_svgf_compat(int W, int H, float *result, float *filtered, void *prev, void *cur, int frame);
/* Selects the argument order of SamplePointOnTriangle's two random numbers
 * (1 = right to left, the reference host build's order). */
void orc_set_point_arg_order(int rtl);

#ifdef __cplusplus
}
#endif
#endif
