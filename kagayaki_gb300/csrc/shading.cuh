// shading.cuh - device-side materials, lights and sampling for the
// wavefront path tracer.
//
// Two estimators share this code:
//  * compat: the reference's RayTrace (RayTrace.cuh:9-109) with its random
//    stream (struct_Xorshift.cuh), Russian roulette
//    (RayTrace_Russian_Roulette.cuh:4-36), NEE to face lights and the
//    environment (NextEventEstimation_FaceLight.cuh:47-120,
//    NextEventEstimation_HDR.cuh:4-58), environment mapping
//    (ImageBasedLighting.cuh:6-91), Lambert and Disney sampling
//    (LambertBRDF_sampling.cuh, Disney_BRDF_sampling.cuh, sampling.cuh).
//  * unbiased: the same BRDF model evaluated with consistent sampling pdfs,
//    a 2D environment CDF sampled inside the texel, balance-heuristic MIS.
#pragma once

#include "kgk_device.cuh"
#include "kgk_internal.h"

namespace kgk {

constexpr float kPI = 3.14159265358979323846f;
constexpr float kSINF = 1e-4f;  // sINF, global_values.cuh:9

// ---------------------------------------------------------------------------
// Random numbers
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long xorshift64(unsigned long long s) {
    if (s == 0ull) s = 1ull;  // struct_Xorshift.cuh:11-14
    s ^= s << 5;
    s ^= s >> 41;
    s ^= s << 20;
    return s;
}

// random_rangeMinMax (struct_Xorshift.cuh:23-31) with the host build's
// rounding: u64 -> float round-to-nearest, no contracted multiply-add.
__device__ __forceinline__ float rnd_ref(unsigned long long &s, float lo, float hi) {
    s = xorshift64(s);
    const float mid = __fmul_rn(__fadd_rn(hi, lo), 0.5f);
    const float r = __fmul_rn(__fsub_rn(hi, lo), 0.5f);
    float ret = __fdiv_rn(__ull2float_rn(s), 18446744073709551616.0f);
    ret = __fmul_rn(2.0f, __fsub_rn(ret, 0.5f));
    return __fadd_rn(__fmul_rn(r, ret), mid);
}

// Unbiased stream: uniform in [0, 1) from the top 24 bits.
__device__ __forceinline__ float rnd_u(unsigned long long &s) {
    s = xorshift64(s);
    return (float)(unsigned)(s >> 40) * (1.0f / 16777216.0f);
}

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// ---------------------------------------------------------------------------
// Frames
// ---------------------------------------------------------------------------
// GenerateONBFromNormal (struct_Vec.cuh:81-86).
__device__ __forceinline__ void onb_ref(float3 n, float3 &u, float3 &v, float3 &w) {
    w = n;
    if (fabsf(w.x) > 1e-4) u = normalize3(cross3(f3(0.0f, 1.0f, 0.0f), w));
    else u = normalize3(cross3(f3(1.0f, 0.0f, 0.0f), w));
    v = normalize3(cross3(w, u));
}

// ---------------------------------------------------------------------------
// Disney BRDF (Disney_BRDF.cuh), evaluated exactly as the reference writes it.
// ---------------------------------------------------------------------------
struct DisneyParams {
    float ax, ay, ac, a_sheen;
    float wt[5];
};

__device__ __forceinline__ DisneyParams disney_params(const kgk_material &m) {
    DisneyParams p;
    const float aspect = sqrtf(1.0f - 0.9f * m.anisotropic);   // RayTrace.cuh:85-89
    p.a_sheen = m.roughness * m.roughness;
    p.ax = fmaxf(0.001f, m.roughness * m.roughness / aspect);
    p.ay = fmaxf(0.001f, m.roughness * m.roughness * aspect);
    p.ac = (1.0f - m.cloearcoatGloss) * 0.1f + m.cloearcoatGloss * 0.001f;
    p.wt[0] = (1.0f - m.subsurface) * (1.0f - m.metallic);     // Disney_BRDF.cuh:9-21
    p.wt[1] = m.subsurface * (1.0f - m.metallic);
    p.wt[2] = 1.0f - m.metallic;
    p.wt[3] = 1.0f;
    p.wt[4] = 1.0f;
    return p;
}

__device__ __forceinline__ float pow5(float x) { return x * x * x * x * x; }
__device__ __forceinline__ float schlick_w(float u) { float m = 1.0f - u; return pow5(m); }

__device__ __forceinline__ float d_gtr2(float3 h, float ax, float ay, float3 u, float3 v, float3 w) {
    const float hu = dot3(h, u), hv = dot3(h, v), hw = dot3(h, w);
    const float q = (hu * hu) / (ax * ax) + (hv * hv) / (ay * ay) + hw * hw;
    return 1.0f / (kPI * ax * ay * q * q);
}

__device__ __forceinline__ float d_berry(float3 h, float3 n, float alpha) {
    alpha = fminf(fmaxf(alpha, 0.0001f), 0.9999f);
    const float a2 = alpha * alpha;
    const float c = fabsf(dot3(h, n));
    return ((a2 - 1.0f) / (2.0f * kPI * logf(alpha))) / ((a2 - 1.0f) * c * c + 1.0f);
}

__device__ __forceinline__ float g_lambda(float3 w, float3 h, float ax, float ay) {
    float3 wx, wy, wz;
    onb_ref(h, wx, wy, wz);
    const float a = dot3(wx, w), b = dot3(wy, w), c = dot3(wz, w);
    return 0.5f * (-1.0f + sqrtf(1.0f + (ax * ax * a * a + ay * ay * b * b) / (c * c)));
}

__device__ __forceinline__ float smith_g(float ndv, float ag) {
    const float a = ag * ag, b = ndv * ndv;
    return 1.0f / (ndv + sqrtf(a + b - a * b));
}

// Smith Lambda of anisotropic GGX in the shading frame (u, v, n).
__device__ __forceinline__ float g_lambda_n(float3 wd, float3 u, float3 v, float3 n, float ax, float ay) {
    const float a = dot3(wd, u), b = dot3(wd, v), c = dot3(wd, n);
    return 0.5f * (-1.0f + sqrtf(1.0f + (ax * ax * a * a + ay * ay * b * b) / (c * c)));
}

// evaluate_Disney_BRDF (Disney_BRDF.cuh:118-133): out = toward the light,
// in = toward the viewer; both leave the surface.
// kRefG = true: the reference's specular shadowing term, whose Lambda is taken
// in a frame built around the half vector (so it does not fall off at grazing
// view or light directions; compat mode reproduces it).  kRefG = false (the
// unbiased estimator): height-correlated Smith G with Lambda in the shading
// frame, which bounds the sampling weight f cos / pdf at grazing angles.
template <bool kRefG = true>
__device__ float3 disney_eval(const kgk_material &m, const DisneyParams &p, float3 out, float3 in,
                              float3 n, float3 u, float3 v, float3 w) {
    if (dot3(n, in) < 0.0f || dot3(n, out) < 0.0f) return f3(0.0f, 0.0f, 0.0f);
    const float3 dif = f3(m.diffuse.x, m.diffuse.y, m.diffuse.z);
    const float3 h = normalize3(out + in);
    const float ndi = dot3(n, in), ndo = dot3(n, out);
    const float FL = schlick_w(ndi), FV = schlick_w(ndo);
    const float hdi = dot3(h, in);
    float3 b = f3(0.0f, 0.0f, 0.0f);
    // diffuse
    {
        const float fd90 = 0.5f + 2.0f * m.roughness * fabsf(hdi) * fabsf(hdi);
        const float fd = ((1.0f - FL) + FL * fd90) * ((1.0f - FV) + FV * fd90);
        b += (dif / kPI) * (fd * p.wt[0]);
    }
    // subsurface
    if (p.wt[1] != 0.0f) {
        const float f90 = m.roughness * hdi * hdi;
        const float fss = ((1.0f - FL) + FL * f90) * ((1.0f - FV) + FV * f90);
        b += (dif / kPI) * (1.25f * (fss * (1.0f / (ndi + ndo) - 0.5f) + 0.5f) * p.wt[1]);
    }
    const float3 nd = normalize3(dif);
    // sheen
    if (m.sheen != 0.0f && p.wt[2] != 0.0f) {
        const float3 rho = f3(1.0f, 1.0f, 1.0f) * (1.0f - m.sheenTint) + nd * m.sheenTint;
        b += rho * (m.sheen * pow5(1.0f - hdi) * p.wt[2]);
    }
    // specular (GTR2 anisotropic, height-correlated-style G of the reference)
    {
        const float3 rho = f3(1.0f, 1.0f, 1.0f) * (1.0f - m.specularTint) + nd * m.specularTint;
        const float3 f0 = rho * ((1.0f - m.metallic) * 0.08f * m.specular) + dif * m.metallic;
        const float fw = pow5(1.0f - dot3(h, n));
        const float3 F = f0 + (f3(1.0f, 1.0f, 1.0f) - f0) * fw;
        const float D = d_gtr2(h, p.ax, p.ay, u, v, w);
        const float G = kRefG ? 1.0f / (1.0f + g_lambda(in, h, p.ax, p.ay) + g_lambda(out, h, p.ax, p.ay))
                              : 1.0f / (1.0f + g_lambda_n(in, u, v, w, p.ax, p.ay) +
                                        g_lambda_n(out, u, v, w, p.ax, p.ay));
        b += F * (D * G / (4.0f * fabsf(ndi) * fabsf(ndo)) * p.wt[3]);
    }
    // clearcoat (GTR1 + Smith 0.25)
    if (m.clearcoat != 0.0f) {
        const float fw = pow5(1.0f - dot3(h, n));
        const float F = 0.04f + 0.96f * fw;
        b += f3(1.0f, 1.0f, 1.0f) * (0.25f * m.clearcoat * F * d_berry(h, n, p.ac) * smith_g(ndi, 0.25f) *
                                     smith_g(ndo, 0.25f) * p.wt[4]);
    }
    return b;
}

// evaluate_Disney_BRDF_pdf (Disney_BRDF.cuh:168-183): the reference's mixture,
// whose specular terms divide by 4|n.out| (not the half-vector Jacobian).
static __device__ float disney_pdf_ref(const DisneyParams &p, float3 in, float3 out, float3 n, float3 u,
                                float3 v, float3 w) {
    const float3 h = normalize3(out + in);
    const float sw = p.wt[0] + p.wt[1] + p.wt[2] + p.wt[3] + p.wt[4];
    float pdf = (p.wt[0] + p.wt[1] + p.wt[2]) * (fmaxf(dot3(n, out), 0.0f) / kPI);
    pdf += p.wt[3] * (d_gtr2(h, p.ax, p.ay, u, v, w) * fabsf(dot3(n, h)) / (4.0f * fabsf(dot3(n, out))));
    pdf += p.wt[4] * (d_berry(h, n, p.ac) * fabsf(dot3(n, h)) / (4.0f * fabsf(dot3(n, out))));
    return pdf / sw;
}

// Consistent mixture pdf of disney_sample_unbiased: lobe probabilities wt/sum,
// half-vector Jacobian 1 / (4 |out.h|).
static __device__ float disney_pdf_unbiased(const DisneyParams &p, float3 in, float3 out, float3 n, float3 u,
                                     float3 v, float3 w) {
    const float ndo = dot3(n, out);
    if (ndo <= 0.0f || dot3(n, in) <= 0.0f) return 0.0f;
    const float3 h = normalize3(out + in);
    const float ohd = fabsf(dot3(out, h));
    const float nh = fabsf(dot3(n, h));
    const float sw = p.wt[0] + p.wt[1] + p.wt[2] + p.wt[3] + p.wt[4];
    float pdf = (p.wt[0] + p.wt[1] + p.wt[2]) * (ndo / kPI);
    pdf += p.wt[3] * d_gtr2(h, p.ax, p.ay, u, v, w) * nh / (4.0f * ohd);
    pdf += p.wt[4] * d_berry(h, n, p.ac) * nh / (4.0f * ohd);
    return pdf / sw;
}

// sample_ray_cosine_weighted (LambertBRDF_sampling.cuh:10-29).
__device__ __forceinline__ float3 sample_cos_ref(unsigned long long &s, float3 u, float3 v, float3 w) {
    const float R1 = rnd_ref(s, 0.0f, 1.0f);
    const float R2 = rnd_ref(s, 0.0f, 0.9999f);
    const float theta = acosf(sqrtf(1.0f - R2));
    const float phi = 2.0f * kPI * R1;
    return normalize3(u * (sinf(theta) * cosf(phi)) + v * (sinf(theta) * sinf(phi)) + w * cosf(theta));
}

__device__ __forceinline__ float3 sample_cos_u(float r1, float r2, float3 u, float3 v, float3 w) {
    const float rr = sqrtf(r2), phi = 2.0f * kPI * r1;
    return normalize3(u * (rr * cosf(phi)) + v * (rr * sinf(phi)) + w * sqrtf(fmaxf(0.0f, 1.0f - r2)));
}

__device__ __forceinline__ float3 reflect_ref(float3 d, float3 h) { return normalize3(d - h * (2.0f * dot3(d, h))); }

// GTR2 anisotropic half vector (Disney_BRDF_sampling.cuh:4-9) from r1, r2.
__device__ __forceinline__ float3 gtr2_half(float R1, float R2, float3 u, float3 v, float3 w, float ax, float ay) {
    const float3 a = u * (ax * cosf(2.0f * kPI * R1)) + v * (ay * sinf(2.0f * kPI * R1));
    return normalize3(a * sqrtf(R2 / (1.0f - R2)) + w);
}

// GTR1 half vector.  The reference takes sin(phi) = +sqrt(1 - cos^2(phi))
// (Disney_BRDF_sampling.cuh:23-30); `full_circle` restores the sign.
__device__ __forceinline__ float3 gtr1_half(float R1, float R2, float3 u, float3 v, float3 w, float alpha,
                                            bool full_circle) {
    const float cphi = cosf(2.0f * kPI * R1);
    float sphi = sqrtf(fmaxf(0.0f, 1.0f - cphi * cphi));
    if (full_circle) sphi = sinf(2.0f * kPI * R1);
    alpha = fminf(fmaxf(alpha, -0.9999f), 0.9999f);
    const float ct = sqrtf((1.0f - powf(alpha, 2.0f * (1.0f - R2))) / (1.0f - alpha * alpha));
    const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
    return u * (st * cphi) + v * (st * sphi) + w * ct;
}

// lower_bound (Algorithms.cuh:6-20): first index with a[i] >= k, or n-1.
__device__ __forceinline__ int lower_bound_f(const float *a, int n, float k) {
    int ng = -1, ok = n - 1;
    while (ok - ng > 1) {
        const int mid = (ok + ng) / 2;
        if (__ldg(&a[mid]) >= k) ok = mid;
        else ng = mid;
    }
    return ok;
}

// Unbiased CDF search over c[0..n] (c[0] = 0, c[n] = 1): k with c[k] <= u < c[k+1].
__device__ __forceinline__ int cdf_search(const float *c, int n, float u) {
    int lo = 0, hi = n;  // invariant c[lo] <= u < c[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&c[mid]) <= u) lo = mid;
        else hi = mid;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// Environment, reference mapping (ImageBasedLighting.cuh)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 uv_sphere_ref(float3 d) {
    float theta;
    const float phi = asinf(d.z);
    if ((double)fabsf(d.z) >= 1.0 - (double)kSINF) theta = 0.0f;
    else if (fabsf(d.x) <= kSINF) theta = d.y > 0.0f ? kPI / 2 : -kPI / 2;
    else {
        const float s = asinf(d.y / sqrtf(1.0f - d.z * d.z));
        if (d.x > 0.0f) theta = s;
        else if (d.x < 0.0f && d.y > 0.0f) theta = kPI - s;
        else theta = -1.0f * kPI - s;
    }
    return make_float2(fminf(fmaxf(theta / (2.0f * kPI) + 0.5f, 0.0f), 1.0f),
                       fminf(fmaxf(phi / kPI + 0.5f, 0.0f), 1.0f));
}

__device__ __forceinline__ float3 env_texel(const DevScene &s, int idx) {
    const float *p = s.env + (size_t)idx * s.env_bpp;
    return f3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}

// get_HDR_emission (ImageBasedLighting.cuh:33-44).
__device__ __forceinline__ float3 env_lookup_ref(const DevScene &s, float3 d) {
    const float2 uv = uv_sphere_ref(d);
    int idx = s.env_w * (int)((float)(s.env_h - 1) * (1.0f - uv.y)) + (int)((float)(s.env_w - 1) * (1.0f - uv.x));
    idx = min(max(idx, 0), s.env_w * s.env_h - 1);
    return env_texel(s, idx);
}

// calculate_HDR_pdf (ImageBasedLighting.cuh:83-91); the index is clamped where
// the reference would read one past the end (direction exactly -z).
__device__ __forceinline__ float env_pdf_ref(const DevScene &s, float3 d) {
    const float2 uv = uv_sphere_ref(d);
    int idx = s.env_w * (int)((float)s.env_h * (1.0f - uv.y)) + (int)((float)s.env_w * uv.x);
    const int n = s.env_w * s.env_h;
    idx = min(max(idx, 0), n - 1);
    const float tot = __ldg(&s.env_cdf_ref[n - 1]);
    if (idx == 0) return __ldg(&s.env_cdf_ref[0]) / tot;
    return (__ldg(&s.env_cdf_ref[idx]) - __ldg(&s.env_cdf_ref[idx - 1])) / tot;
}

// convert_HDRindex_to_Dir (ImageBasedLighting.cuh:46-56): texel corner direction.
__device__ __forceinline__ float3 env_index_to_dir_ref(const DevScene &s, int index, float &pdf) {
    const float u = 1.0f - (float)(index % s.env_w) / (float)s.env_w;
    const float v = 1.0f - (float)(index / s.env_w) / (float)s.env_h;
    const float theta = (u - 0.5f) * 2.0f * kPI;
    const float phi = (v - 0.5f) * kPI;
    const float cp = cosf(phi);
    if (fabsf(cp) < kSINF) pdf *= 1.0f / (2.0f * kPI * kPI * kSINF);
    else pdf *= 1.0f / (2.0f * kPI * kPI * cp);
    pdf *= (float)(s.env_w * s.env_h);
    return f3(cp * cosf(theta), cp * sinf(theta), sinf(phi));
}

// ---------------------------------------------------------------------------
// Environment, unbiased: the same lat-long layout (row 0 = +z, column c at
// u = 1 - c/W), piecewise-constant radiance, pdf over solid angle.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void env_dir_to_texel(const DevScene &s, float3 d, int &row, int &col, float &cosl) {
    const float z = fminf(fmaxf(d.z, -1.0f), 1.0f);
    const float phi = asinf(z);                          // latitude
    const float theta = atan2f(d.y, d.x);                // longitude in (-pi, pi]
    const float v = phi / kPI + 0.5f;                     // 1 at +z
    const float u = theta / (2.0f * kPI) + 0.5f;
    row = min(max((int)((1.0f - v) * s.env_h), 0), s.env_h - 1);
    col = min(max((int)((1.0f - u) * s.env_w), 0), s.env_w - 1);
    cosl = cosf(phi);
}

__device__ __forceinline__ float env_texel_weight(const DevScene &s, int row, int col) {
    return __ldg(&s.env_prob[(size_t)row * s.env_w + col]);  // probability of the texel
}

// Solid-angle pdf of direction d under env importance sampling: the texel's
// probability spread uniformly over (longitude, latitude) inside the texel,
// divided by the solid-angle element cos(latitude) of d itself.
__device__ __forceinline__ float env_pdf_u(const DevScene &s, float3 d) {
    int row, col;
    float cosl;
    env_dir_to_texel(s, d, row, col, cosl);
    if (cosl <= 1e-7f) return 0.0f;
    return env_texel_weight(s, row, col) * (float)s.env_w * (float)s.env_h / (2.0f * kPI * kPI * cosl);
}

__device__ __forceinline__ float3 env_lookup_u(const DevScene &s, float3 d) {
    int row, col;
    float cosl;
    env_dir_to_texel(s, d, row, col, cosl);
    return env_texel(s, row * s.env_w + col);
}

// Samples a direction; returns it with its solid-angle pdf and radiance.
// Inside the texel the direction is uniform in (longitude, latitude), so its
// solid-angle density carries 1 / cos(latitude) of the sampled direction.
// The texel comes from the alias table: a uniform index (from 64 random
// bits, so every index is equally likely to within 2^-40) and one coin.
__device__ __forceinline__ float3 env_sample_u(const DevScene &s, unsigned long long &rs, float &pdf, float3 &Le) {
    const unsigned long long n = (unsigned long long)s.env_w * (unsigned long long)s.env_h;
    rs = xorshift64(rs);
    int t = (int)__umul64hi(rs, n);
    const float coin = rnd_u(rs), r2 = rnd_u(rs), r3 = rnd_u(rs);
    const float2 e = __ldg(&s.env_alias[t]);
    if (coin >= e.x) t = __float_as_int(e.y);
    const int row = t / s.env_w, col = t - row * s.env_w;
    const float v = 1.0f - (row + r2) / s.env_h;
    const float u = 1.0f - (col + r3) / s.env_w;
    const float phi = (v - 0.5f) * kPI, theta = (u - 0.5f) * 2.0f * kPI;
    const float cp = cosf(phi);
    const float3 d = f3(cp * cosf(theta), cp * sinf(theta), sinf(phi));
    pdf = cp > 1e-7f ? env_texel_weight(s, row, col) * (float)s.env_w * (float)s.env_h / (2.0f * kPI * kPI * cp)
                     : 0.0f;
    Le = env_texel(s, row * s.env_w + col);
    return d;
}

// ---------------------------------------------------------------------------
// Textures: nearest fetch (Texture::get_Color, struct_Texture.cuh:12-18;
// the index is clamped where the reference reads past the end, v = 0) or
// bilinear; float or RGBA8 texels.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float3 tex_texel(const DevScene &s, const TexDesc &td, int idx) {
    if (td.rgba8) {
        const uchar4 b = __ldg(&s.tex_rgba8[td.offset + idx]);
        return f3(__ldg(&s.tex_lut[b.x]), __ldg(&s.tex_lut[b.y]), __ldg(&s.tex_lut[b.z]));
    }
    // three consecutive floats from the texel, as Texture::get_Color reads
    // them: with fewer than 3 channels they run into the next texels (the
    // reference's behaviour); clamped at the end of the texture
    const int n_el = td.w * td.h * td.bpp;
    const int e = idx * td.bpp;
    const float *p = s.tex_pixels + td.offset;
    return f3(__ldg(p + e), __ldg(p + min(e + 1, n_el - 1)), __ldg(p + min(e + 2, n_el - 1)));
}

__device__ __forceinline__ float3 tex_fetch(const DevScene &s, int tex, float u, float v) {
    const TexDesc td = s.tex[tex];
    if (s.tex_filter == 1) {
        // bilinear, texel centres at (i + 0.5) / w, wrap-around addressing
        const float x = u * td.w - 0.5f, y = (1.0f - v) * td.h - 0.5f;
        const float fx = floorf(x), fy = floorf(y);
        const float ax = x - fx, ay = y - fy;
        int x0 = (int)fx % td.w, y0 = (int)fy % td.h;
        if (x0 < 0) x0 += td.w;
        if (y0 < 0) y0 += td.h;
        const int x1 = x0 + 1 == td.w ? 0 : x0 + 1, y1 = y0 + 1 == td.h ? 0 : y0 + 1;
        const float3 c00 = tex_texel(s, td, y0 * td.w + x0), c10 = tex_texel(s, td, y0 * td.w + x1);
        const float3 c01 = tex_texel(s, td, y1 * td.w + x0), c11 = tex_texel(s, td, y1 * td.w + x1);
        return (c00 * (1.0f - ax) + c10 * ax) * (1.0f - ay) + (c01 * (1.0f - ax) + c11 * ax) * ay;
    }
    int idx = td.w * (int)((float)td.h * (1.0f - v)) + (int)((float)td.w * u);
    idx = min(max(idx, 0), td.w * td.h - 1);
    return tex_texel(s, td, idx);
}

}  // namespace kgk
