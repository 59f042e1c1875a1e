// traverse.cuh - closest-hit and occlusion traversal of the 8-wide
// compressed BVH with watertight FP32 ray/triangle intersection.
// Replaces willIntersectWithTriangle_nonRecursive (ConstructBVH.cuh:286-368)
// and Triangle::intersectTest (struct_Triangle.cuh:30-79) on the device.
//
// Semantics kept from the reference: a hit needs t >= 1e-5 (double compare,
// struct_Triangle.cuh:57), the result is the closest hit, and the reported
// distance is computed by the reference's own expression (ref_distance).  Where the
// reference resolves equal distances by its traversal order, this resolves
// them to the smaller triangle id, independent of the tree.
// Differences by design: the test is watertight (Woop, Benthin, Wald 2013)
// instead of Cramer's rule, and node culling uses the ray's [tmin, tmax]
// interval (closest-hit pruning) instead of the whole line.
#pragma once

#include "kgk_device.cuh"
#include "kgk_internal.h"

namespace kgk {

constexpr int kTravStack = 32;
// Node visits a resumable traversal step may make before it tests triangles
// (the closest-hit rays of k_extend and the batch queries; the shadow passes).
constexpr int kNodesPerStep = 2;
constexpr int kNodesPerStepShadow = 2;
// Conservative widening of box exit distances: 1 + 2 * gamma(5) covers the
// rounding of the origin offset, the multiply, the two roundings of the
// biased plane offset and the plane's multiply-add.
constexpr float kBoxWiden = 1.0000006f;

struct RayPre {
    float3 o, d, inv;
    float sx, sy, sz;
    int kx, ky, kz;
    unsigned oct_inv4;
};

__device__ __forceinline__ float safe_inv(float d) {
    // |d| < 1e-20 -> +-1e20 so that scale * inv never forms 0 * inf
    float a = fabsf(d) < 1e-20f ? copysignf(1e-20f, d) : d;
    return 1.0f / a;
}

__device__ __forceinline__ RayPre make_ray(float3 o, float3 d) {
    RayPre r;
    r.o = o;
    r.d = d;
    r.inv = f3(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = ax > ay ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz == 2 ? 0 : kz + 1;
    int ky = kx == 2 ? 0 : kx + 1;
    if (comp(d, kz) < 0.0f) { int t = kx; kx = ky; ky = t; }
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    const float dz = comp(d, kz);
    r.sx = comp(d, kx) / dz;
    r.sy = comp(d, ky) / dz;
    r.sz = 1.0f / dz;
    unsigned oct = (d.x < 0.0f ? 4u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 1u : 0u);
    r.oct_inv4 = (7u - oct) * 0x01010101u;
    return r;
}

// Watertight test.  On a hit returns true with t, b1 (weight of v1) and b2
// (weight of v2).  The 2D edge functions are formed with explicit
// round-to-nearest multiplies and subtractions (no FMA contraction), so the
// two triangles sharing an edge compute exactly negated values.
__device__ __forceinline__ bool tri_intersect(const RayPre &r, float4 a4, float4 b4, float4 c4,
                                              float *t, float *b1, float *b2) {
    const float3 A = f3(a4) - r.o, B = f3(b4) - r.o, C = f3(c4) - r.o;
    const float Akz = comp(A, r.kz), Bkz = comp(B, r.kz), Ckz = comp(C, r.kz);
    const float Ax = comp(A, r.kx) - r.sx * Akz, Ay = comp(A, r.ky) - r.sy * Akz;
    const float Bx = comp(B, r.kx) - r.sx * Bkz, By = comp(B, r.ky) - r.sy * Bkz;
    const float Cx = comp(C, r.kx) - r.sx * Ckz, Cy = comp(C, r.ky) - r.sy * Ckz;
    const float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    const float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    const float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = U + V + W;
    if (det == 0.0f) return false;
    const float T = U * (r.sz * Akz) + V * (r.sz * Bkz) + W * (r.sz * Ckz);
    const float tt = T / det;
    if (!(tt >= kTMin)) return false;  // also rejects NaN
    *t = tt;
    *b1 = V / det;
    *b2 = W / det;
    return true;
}

// Distance and barycentrics of an accepted hit by the reference's own
// expressions (struct_Triangle.cuh:46-49), every operation rounded
// separately like the reference's host build: the reported t is the
// reference's t bit for bit.  u = weight of v1, v = weight of v2.
__device__ __forceinline__ float3 rn_sub(float3 a, float3 b) {
    return f3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}
__device__ __forceinline__ float3 rn_cross(float3 a, float3 b) {
    return f3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
              __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
              __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float rn_dot(float3 a, float3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ void ref_distance(const RayPre &r, float4 a4, float4 b4, float4 c4, float *t, float *u,
                                             float *v) {
    const float3 v0 = f3(a4), e1 = rn_sub(f3(b4), v0), e2 = rn_sub(f3(c4), v0), so = rn_sub(r.o, v0);
    const float3 de2 = rn_cross(r.d, e2), se1 = rn_cross(so, e1);
    const float term1 = __fdiv_rn(1.0f, rn_dot(de2, e1));
    *t = __fmul_rn(term1, rn_dot(se1, e2));
    *u = __fmul_rn(term1, rn_dot(de2, so));
    *v = __fmul_rn(term1, rn_dot(se1, r.d));
}

__device__ __forceinline__ unsigned byte_of(unsigned x, int i) { return (x >> (i * 8)) & 0xffu; }
// 2^15 + (byte i of x) as a float, exactly, in one byte permute: the byte
// becomes mantissa bits 8..15 under the exponent of 2^15 (bits 0x47000000).
// The box test folds the bias into its per-node plane offsets, so a plane
// costs one permute and one multiply-add (no integer-to-float conversion and
// no subtraction).
__device__ __forceinline__ float byte_biased(unsigned x, int i) {
    return __uint_as_float(__byte_perm(x, 0x4700u, 0x5404u | ((unsigned)i << 4)));
}
__device__ __forceinline__ unsigned sign_extend_s8x4(unsigned x) { return ((x >> 7) & 0x01010101u) * 0xffu; }

// Child hit mask of one compressed node: bits 24..31 = inner children
// (octant-permuted slots), bits 0..23 = triangles of hit leaf children.
__device__ __forceinline__ unsigned node_intersect(const RayPre &r, float tmin, float tmax,
                                                   const float4 n0, const float4 n1, const float4 n2,
                                                   const float4 n3, const float4 n4) {
    const unsigned e = __float_as_uint(n0.w);
    const float adx = __uint_as_float((e & 0xffu) << 23) * r.inv.x;
    const float ady = __uint_as_float(((e >> 8) & 0xffu) << 23) * r.inv.y;
    const float adz = __uint_as_float(((e >> 16) & 0xffu) << 23) * r.inv.z;
    // Plane b of an axis lies at t = (2^15 + b) * ad + (o - 2^15 * ad),
    // formed as one multiply-add with an exact product.  The offset is
    // rounded twice (o - 2^15 ad, then -/+ the slack), each time by at most
    // 2^-24 (|o| + 2^15 |ad|) = 2^-24 |o| + 2^-9 |ad|.  A slack of 1/64 of the
    // axis's quantum (|ad| / 64: per axis, since |ad| is huge on an axis the
    // ray nearly parallels) moves near planes down and far planes up, four
    // times the |ad| parts; kBoxWiden covers the |o| parts.
    const float ox = (n0.x - r.o.x) * r.inv.x;
    const float oy = (n0.y - r.o.y) * r.inv.y;
    const float oz = (n0.z - r.o.z) * r.inv.z;
    const float bx = fmaf(-32768.0f, adx, ox), by = fmaf(-32768.0f, ady, oy), bz = fmaf(-32768.0f, adz, oz);
    const float sx = fabsf(adx) * 0.015625f, sy = fabsf(ady) * 0.015625f, sz = fabsf(adz) * 0.015625f;
    const float oxn = bx - sx, oyn = by - sy, ozn = bz - sz;
    const float oxf = bx + sx, oyf = by + sy, ozf = bz + sz;
    const float tm = tmax * kBoxWiden;
    unsigned hits = 0;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const unsigned meta4 = __float_as_uint(half ? n1.w : n1.z);
        const unsigned is_inner4 = (meta4 & (meta4 << 1)) & 0x10101010u;
        const unsigned inner_mask4 = sign_extend_s8x4(is_inner4 << 3);
        const unsigned bit_index4 = (meta4 ^ (r.oct_inv4 & inner_mask4)) & 0x1f1f1f1fu;
        const unsigned child_bits4 = (meta4 >> 5) & 0x07070707u;
        const unsigned qlx = __float_as_uint(half ? n2.y : n2.x), qhx = __float_as_uint(half ? n2.w : n2.z);
        const unsigned qly = __float_as_uint(half ? n3.y : n3.x), qhy = __float_as_uint(half ? n3.w : n3.z);
        const unsigned qlz = __float_as_uint(half ? n4.y : n4.x), qhz = __float_as_uint(half ? n4.w : n4.z);
        const unsigned xn = r.d.x < 0.0f ? qhx : qlx, xf = r.d.x < 0.0f ? qlx : qhx;
        const unsigned yn = r.d.y < 0.0f ? qhy : qly, yf = r.d.y < 0.0f ? qly : qhy;
        const unsigned zn = r.d.z < 0.0f ? qhz : qlz, zf = r.d.z < 0.0f ? qlz : qhz;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float t0x = fmaf(byte_biased(xn, j), adx, oxn);
            const float t0y = fmaf(byte_biased(yn, j), ady, oyn);
            const float t0z = fmaf(byte_biased(zn, j), adz, ozn);
            const float t1x = fmaf(byte_biased(xf, j), adx, oxf);
            const float t1y = fmaf(byte_biased(yf, j), ady, oyf);
            const float t1z = fmaf(byte_biased(zf, j), adz, ozf);
            const float lo = fmaxf(fmaxf(t0x, t0y), fmaxf(t0z, tmin));
            const float hi = fminf(fminf(t1x, t1y), fminf(t1z, tm)) * kBoxWiden;
            if (lo <= hi) hits |= byte_of(child_bits4, j) << byte_of(bit_index4, j);
        }
    }
    return hits;
}

struct TravStats {
    unsigned nodes, tris, overflow;
};

// Closest hit.  best_t in: search limit (exclusive of farther hits); out: hit
// distance.  Returns the BVH-order triangle index of the hit or -1.
// Both traversals check every node and triangle index against the buffer
// sizes; a bad index sets st.overflow = 2 and ends the traversal instead of
// reading out of range.
template <bool kCount>
__device__ __forceinline__ int trace_closest(const WideNode *__restrict__ nodes, unsigned n_nodes,
                                             const float4 *__restrict__ tri, unsigned n_tris,
                                             const RayPre &r, float &best_t, int &best_id, float &bu,
                                             float &bv, TravStats &st) {
    uint2 stack[kTravStack];
    int sp = 0;
    int hit_slot = -1;
    uint2 group = make_uint2(0u, 0x80000000u);
    while (true) {
        uint2 tg = make_uint2(0u, 0u);
        if (group.y & 0xff000000u) {
            const unsigned hits_imask = group.y;
            const int child_bit = 31 - __clz(hits_imask & 0xff000000u);
            const unsigned base = group.x;
            group.y &= ~(1u << child_bit);
            if (group.y & 0xff000000u) {
                if (sp < kTravStack) stack[sp++] = group;
                else st.overflow = 1;
            }
            const unsigned slot = (unsigned)(child_bit - 24) ^ (r.oct_inv4 & 0xffu);
            const unsigned rel = __popc(hits_imask & ~(0xffffffffu << slot));
            if (base + rel >= n_nodes) { st.overflow = 2; break; }
            const WideNode *nd = nodes + base + rel;
            const float4 n0 = __ldg(&nd->n0), n1 = __ldg(&nd->n1), n2 = __ldg(&nd->n2),
                         n3 = __ldg(&nd->n3), n4 = __ldg(&nd->n4);
            if (kCount) ++st.nodes;
            const unsigned hm = node_intersect(r, 0.0f, best_t, n0, n1, n2, n3, n4);
            const unsigned imask = __float_as_uint(n0.w) >> 24;
            group = make_uint2(__float_as_uint(n1.x), (hm & 0xff000000u) | imask);
            tg = make_uint2(__float_as_uint(n1.y), hm & 0x00ffffffu);
        } else {
            tg = group;
            group = make_uint2(0u, 0u);
        }
        while (tg.y != 0u) {
            const int k = __ffs(tg.y) - 1;
            tg.y &= tg.y - 1u;
            const int ti = (int)tg.x + k;
            if ((unsigned)ti >= n_tris) { st.overflow = 2; tg.y = 0u; group = make_uint2(0u, 0u); sp = 0; break; }
            const float4 a = __ldg(&tri[3 * ti]), b = __ldg(&tri[3 * ti + 1]), c = __ldg(&tri[3 * ti + 2]);
            if (kCount) ++st.tris;
            float t, u, v;
            if (tri_intersect(r, a, b, c, &t, &u, &v)) {
                ref_distance(r, a, b, c, &t, &u, &v);
                if (!(t >= kTMin)) continue;
                const int id = __float_as_int(a.w);
                if (t < best_t || (t == best_t && id < best_id)) {
                    best_t = t;
                    best_id = id;
                    bu = u;
                    bv = v;
                    hit_slot = ti;
                }
            }
        }
        if ((group.y & 0xff000000u) == 0u) {
            if (sp == 0) break;
            group = stack[--sp];
        }
    }
    return hit_slot;
}

// Occlusion: true when any triangle lies at kTMin <= t < tmax.
template <bool kCount>
__device__ __forceinline__ bool trace_any(const WideNode *__restrict__ nodes, unsigned n_nodes,
                                          const float4 *__restrict__ tri, unsigned n_tris,
                                          const RayPre &r, float tmax, TravStats &st) {
    uint2 stack[kTravStack];
    int sp = 0;
    uint2 group = make_uint2(0u, 0x80000000u);
    while (true) {
        uint2 tg = make_uint2(0u, 0u);
        if (group.y & 0xff000000u) {
            const unsigned hits_imask = group.y;
            const int child_bit = 31 - __clz(hits_imask & 0xff000000u);
            const unsigned base = group.x;
            group.y &= ~(1u << child_bit);
            if (group.y & 0xff000000u) {
                if (sp < kTravStack) stack[sp++] = group;
                else st.overflow = 1;
            }
            const unsigned slot = (unsigned)(child_bit - 24) ^ (r.oct_inv4 & 0xffu);
            const unsigned rel = __popc(hits_imask & ~(0xffffffffu << slot));
            if (base + rel >= n_nodes) { st.overflow = 2; break; }
            const WideNode *nd = nodes + base + rel;
            const float4 n0 = __ldg(&nd->n0), n1 = __ldg(&nd->n1), n2 = __ldg(&nd->n2),
                         n3 = __ldg(&nd->n3), n4 = __ldg(&nd->n4);
            if (kCount) ++st.nodes;
            const unsigned hm = node_intersect(r, 0.0f, tmax, n0, n1, n2, n3, n4);
            const unsigned imask = __float_as_uint(n0.w) >> 24;
            group = make_uint2(__float_as_uint(n1.x), (hm & 0xff000000u) | imask);
            tg = make_uint2(__float_as_uint(n1.y), hm & 0x00ffffffu);
        } else {
            tg = group;
            group = make_uint2(0u, 0u);
        }
        while (tg.y != 0u) {
            const int k = __ffs(tg.y) - 1;
            tg.y &= tg.y - 1u;
            const int ti = (int)tg.x + k;
            if ((unsigned)ti >= n_tris) { st.overflow = 2; tg.y = 0u; group = make_uint2(0u, 0u); sp = 0; break; }
            const float4 a = __ldg(&tri[3 * ti]), b = __ldg(&tri[3 * ti + 1]), c = __ldg(&tri[3 * ti + 2]);
            if (kCount) ++st.tris;
            float t, u, v;
            if (tri_intersect(r, a, b, c, &t, &u, &v)) {
                ref_distance(r, a, b, c, &t, &u, &v);
                if (t >= kTMin && t < tmax) return true;
            }
        }
        if ((group.y & 0xff000000u) == 0u) {
            if (sp == 0) break;
            group = stack[--sp];
        }
    }
    return false;
}

// ---------------------------------------------------------------------------
// Resumable traversal, a few node visits per call, for kernels that refill
// finished lanes with new rays (dynamic ray fetch) instead of letting a warp
// wait for its longest ray.  Same node order, culling and hit rules as
// trace_closest / trace_any, so the results are the same.
// ---------------------------------------------------------------------------
// The stack lives in a separate local array (TravStack) so that the scalar
// state stays in registers.
struct TravStack {
    uint2 e[kTravStack];
};
struct Trav {
    uint2 group;
    int sp;
    float best_t, bu, bv;
    int best_id, hit_slot;
};

__device__ __forceinline__ void trav_init(Trav &c, float tmax) {
    c.sp = 0;
    c.group = make_uint2(0u, 0x80000000u);
    c.best_t = tmax;
    c.bu = 0.0f;
    c.bv = 0.0f;
    c.best_id = 0x7fffffff;
    c.hit_slot = -1;
}

// Visits nodes until one has hit leaf triangles (at most kNodesPerStep
// nodes), then tests those triangles: the same order as trace_closest /
// trace_any, in fewer, more even steps.  any_mode: stop at the
// first triangle with kTMin <= t < best_t (occlusion); otherwise keep the
// closest hit (ties to the smaller id).  Returns true when the traversal is
// finished; then c.hit_slot is -1 (no hit) or, for the BVH-order triangle ti
// hit, 2 * ti + its material class (the .w of its second record: 1 = Disney).
template <bool kCount, int kVisits = kNodesPerStep>
__device__ __forceinline__ bool trav_step(const WideNode *__restrict__ nodes, unsigned n_nodes,
                                          const float4 *__restrict__ tri, unsigned n_tris, const RayPre &r,
                                          Trav &c, TravStack &stk, bool any_mode, TravStats &st) {
    uint2 tg = make_uint2(0u, 0u);
#pragma unroll 1
    for (int visit = 0; visit < kVisits && tg.y == 0u; ++visit) {
        if ((c.group.y & 0xff000000u) == 0u) {
            if (c.sp == 0) break;
            c.group = stk.e[--c.sp];
        }
        const unsigned hits_imask = c.group.y;
        const int child_bit = 31 - __clz(hits_imask & 0xff000000u);
        const unsigned base = c.group.x;
        c.group.y &= ~(1u << child_bit);
        if (c.group.y & 0xff000000u) {
            if (c.sp < kTravStack) stk.e[c.sp++] = c.group;
            else st.overflow = 1;
        }
        const unsigned slot = (unsigned)(child_bit - 24) ^ (r.oct_inv4 & 0xffu);
        const unsigned rel = __popc(hits_imask & ~(0xffffffffu << slot));
        if (base + rel >= n_nodes) { st.overflow = 2; return true; }
        const WideNode *nd = nodes + base + rel;
        const float4 n0 = __ldg(&nd->n0), n1 = __ldg(&nd->n1), n2 = __ldg(&nd->n2), n3 = __ldg(&nd->n3),
                     n4 = __ldg(&nd->n4);
        if (kCount) ++st.nodes;
        const unsigned hm = node_intersect(r, 0.0f, c.best_t, n0, n1, n2, n3, n4);
        const unsigned imask = __float_as_uint(n0.w) >> 24;
        c.group = make_uint2(__float_as_uint(n1.x), (hm & 0xff000000u) | imask);
        tg = make_uint2(__float_as_uint(n1.y), hm & 0x00ffffffu);
    }
    while (tg.y != 0u) {
        const int k = __ffs(tg.y) - 1;
        tg.y &= tg.y - 1u;
        const int ti = (int)tg.x + k;
        if ((unsigned)ti >= n_tris) { st.overflow = 2; return true; }
        const float4 a = __ldg(&tri[3 * ti]), b = __ldg(&tri[3 * ti + 1]), cc = __ldg(&tri[3 * ti + 2]);
        if (kCount) ++st.tris;
        float t, u, v;
        if (tri_intersect(r, a, b, cc, &t, &u, &v)) {
            ref_distance(r, a, b, cc, &t, &u, &v);
            if (!(t >= kTMin)) continue;
            const int id = __float_as_int(a.w);
            if (any_mode) {
                if (t < c.best_t) {
                    c.best_t = t;
                    c.best_id = id;
                    c.hit_slot = 2 * ti + __float_as_int(b.w);
                    return true;
                }
            } else if (t < c.best_t || (t == c.best_t && id < c.best_id)) {
                c.best_t = t;
                c.best_id = id;
                c.bu = u;
                c.bv = v;
                c.hit_slot = 2 * ti + __float_as_int(b.w);
            }
        }
    }
    if ((c.group.y & 0xff000000u) == 0u) {
        if (c.sp == 0) return true;
        c.group = stk.e[--c.sp];
    }
    return false;
}

}  // namespace kgk
