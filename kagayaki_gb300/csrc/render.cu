// render.cu - wavefront path tracer.  Replaces the per-pixel megakernel
// render<<<W*H/256, 256>>> (render.cuh:21-49, RayTrace.cuh:9-109).
//
// One wave = one path per (pixel, sample) pair.  The live paths' state sits
// densely in SoA arrays (two buffers, used in turn): slot i of the current
// buffer holds the i-th live path, with its id (pixel + sample * pixels).
// Per bounce:
//   extend  closest hit of every live path, written to hit[slot]; the slot
//           goes to the hit or the miss queue (warp-ballot appends);
//   shade   misses: the sky lookup, the path ends; hits: emission, Russian
//           roulette, next-event estimation (shadow-ray records with their
//           contribution precomputed), BSDF sampling.  A continuing path's
//           state moves to the next buffer at the slot a warp-ballot append
//           gives it, a finished path's radiance goes to fin[id] - so the
//           kernels read and write the state of neighbouring slots together;
//   shadow  two passes (face lights, environment) - at most one record per
//           path per pass, so each adds to its path's radiance (in the next
//           buffer, or in fin) without atomics and in the reference's order
//           (face light, then environment).
// Kernels are persistent grid-stride loops that read their counts from device
// memory: the host only reads the live count between bounces.
#include <cmath>
#include <cstring>
#include <vector>

#include <cooperative_groups.h>

#include "kgk_nrc.h"
#include "kgk_scene.h"
#include "shading.cuh"
#include "traverse.cuh"

namespace kgk {
namespace cg = cooperative_groups;

// Device bytes per path in flight (ensure_wave): two buffers of state (4
// float4, rng, depth, id), the final radiance and the hit (float4 each), the
// miss / Lambert / Disney slot queues, two shadow queues of three float4; with the cache
// also its spread and flags (two buffers) and a query record.
constexpr size_t kPathStateBytes = 2 * (4 * 16 + 8 + 4 + 4) + 2 * 16 + 3 * 4 + 2 * 3 * 16;
constexpr size_t kCachePathBytes = 2 * (8 + 4) + 20 * 4;

// Live path state, one buffer (slot = position among the live paths).
struct PathBuf {
    float4 *o = nullptr;              // origin
    float4 *d = nullptr;              // direction, w: pdf of the sampled direction (0 = no MIS)
    float4 *thr = nullptr;            // throughput
    float4 *rad = nullptr;            // radiance gathered so far
    unsigned long long *rng = nullptr;
    int *depth = nullptr;
    int *id = nullptr;                // path id: pixel + sample * pixels
    float2 *spread = nullptr;         // cache: (sqrt-summed path spread, primary footprint)
    int *pflags = nullptr;            // cache: bit 0 training path, bit 1 queried, bits 8.. suffix bounces
};

struct RenderState {
    cudaStream_t st2 = nullptr;               // the shadow passes, overlapping the next bounce's extend
    cudaEvent_t shaded = nullptr, shadowed = nullptr;
    int W = 0, H = 0;                         // per-pixel buffers
    unsigned long long *seeds = nullptr;      // compat per-pixel seed chain (render.cuh:19,29,42)
    float4 *frame = nullptr;                  // per-call radiance sum
    float4 *kept = nullptr;                   // the output frame kept on the device (kgk_render out == NULL)
    bool kept_valid = false;
    double *acc_sum = nullptr, *acc_sq = nullptr;  // FP64 accumulator (3 per pixel)
    unsigned long long acc_n = 0;
    int acc_W = 0, acc_H = 0;
    // G-buffer of the last frame (SVGF input), per pixel
    float4 *gb_pos = nullptr;   // position, depth (hit distance)
    float4 *gb_nrm = nullptr;   // shading normal toward the camera, object id bits
    float4 *gb_alb = nullptr;   // albedo, material id bits
    float4 *gb_emi = nullptr;   // emission, hit flag
    // wave state (capacity cap paths)
    int cap = 0;
    PathBuf pb[2];                            // live path state, used in turn
    float4 *fin = nullptr;                    // final radiance by path id
    float4 *hit = nullptr;                    // closest hit by slot (t, u, v, triangle id or -1)
    int *mq = nullptr;                        // slots whose ray missed the scene
    int *lq = nullptr, *dq = nullptr;         // slots whose ray hit a Disney / another material
    float4 *sh_o[2] = {nullptr, nullptr}, *sh_d[2] = {nullptr, nullptr}, *sh_c[2] = {nullptr, nullptr};
    int *cnt = nullptr;                       // queue counters
    unsigned long long *stats = nullptr;      // rays_closest, rays_shadow, overflow, nodes, tris
    // radiance cache (capacity cap paths; spread and flags are in pb)
    float *qrec = nullptr;                    // query records, kQRec floats each
    float *trec = nullptr;                    // training records, kQRec floats each
    float *ttgt = nullptr;                    // training targets (3 per record)
    int tcap = 0;
    int qrec_cap = 0;                         // paths the cache arrays above hold
    // deferred tail shadow rays (kDeferSlots slots)
    float4 *td_o = nullptr, *td_d = nullptr, *td_c = nullptr;
    int *td_list = nullptr;
    unsigned *td_mask = nullptr;
    unsigned char *td_vis = nullptr;
    // device bytes held for `cap` paths (they count as available when sizing the wave)
    size_t cap_bytes_held() const { return (size_t)cap * kPathStateBytes + (size_t)qrec_cap * kCachePathBytes; }
    int sms = 0;
    bool gbuffer_valid = false;               // G-buffer written by the last frame
    kgk_camera gbuffer_cam{};
};

namespace {

// Device counters: live paths in each state buffer, shadow-queue sizes,
// dynamic-fetch cursors of the extend and shadow kernels, miss / Lambert /
// Disney queue sizes (zeroed before every bounce together with the shadow
// queues), cache record counts.
enum Cnt {
    kA0 = 0, kA1 = 1, kSH0 = 2, kSH1 = 3, kFE = 4, kFS0 = 5, kFS1 = 6, kMQ = 7, kLQ = 8, kDQ = 9, kQN = 10,
    kTN = 11, kTD = 12, kTDF = 13, kTF = 14, kNCnt = 15
};
// Lanes of a warp that must be idle before the warp fetches new rays.
constexpr int kRefill = 8;

// Cache record: raw query [13], T [3], path id (int bits), radiance before the
// query vertex's scattering [3].
constexpr int kQRec = 20;
enum Stat { kRaysC = 0, kRaysS = 1, kOverflow = 2, kNodes = 3, kTris = 4, kRaysT = 5, kNStat = 8 };
// Paths few enough to finish in the tail kernel (one thread per path).
constexpr int kTailPaths = 1 << 17;
// Idle lanes of a tail warp that take new paths together.
constexpr int kTailRefill = 8;
// Deferred shadow rays of the tail (unbiased estimator without the cache):
// the first kDeferBounces bounces of a tail path leave their face-light and
// environment shadow rays in fixed slots (path, bounce, kind) instead of
// tracing them on the path's chain; a parallel pass traces them and another
// adds the visible contributions in slot order.
constexpr int kDeferBounces = 16;
constexpr size_t kDeferSlots = (size_t)kTailPaths * kDeferBounces * 2;

struct Params {
    DevScene sc;
    kgk_camera cam;
    int W, H, npx;
    int spp_wave;          // samples per pixel in this wave
    int sample_base;       // first sample index of the wave
    int estimator;
    int max_depth;         // <= 0: unlimited
    int rr_start;
    int write_gbuffer;
    int count_work;
    unsigned long long seed;
    int frame_index;
    // state: the bounce's live paths (cur), the next bounce's (nxt)
    PathBuf cur, nxt;
    float4 *fin, *hit;
    unsigned long long *seeds;
    float4 *gb_pos, *gb_nrm, *gb_alb, *gb_emi;
    int *cnt;
    unsigned long long *stats;
    // deferred tail shadow rays (null: traced inline)
    float4 *td_o, *td_d, *td_c;
    int *td_list;
    unsigned *td_mask;
    unsigned char *td_vis;
    // radiance cache
    int use_cache;
    float *qrec, *trec;
    int tcap;
    int train_stride, train_offset, suffix_max;
    float spread_c;
};

// One live path in registers.
struct PathState {
    float3 o, d, T, rad;
    float pdf;                 // of the sampled direction d (0 = no MIS)
    unsigned long long rs;
    int depth, id;
    float2 sp;                 // cache only
    int fl;                    // cache only
};

__device__ __forceinline__ PathState load_path(const PathBuf &b, int i, bool cache) {
    PathState s;
    const float4 o = b.o[i], d = b.d[i], t = b.thr[i], r = b.rad[i];
    s.o = f3(o);
    s.d = f3(d);
    s.pdf = d.w;
    s.T = f3(t);
    s.rad = f3(r);
    s.rs = b.rng[i];
    s.depth = b.depth[i];
    s.id = b.id[i];
    s.sp = cache ? b.spread[i] : make_float2(0.0f, 0.0f);
    s.fl = cache ? b.pflags[i] : 0;
    return s;
}

__device__ __forceinline__ void store_path(const PathBuf &b, int k, const PathState &s, bool cache) {
    b.o[k] = make_float4(s.o.x, s.o.y, s.o.z, 0.0f);
    b.d[k] = make_float4(s.d.x, s.d.y, s.d.z, s.pdf);
    b.thr[k] = make_float4(s.T.x, s.T.y, s.T.z, 0.0f);
    b.rad[k] = make_float4(s.rad.x, s.rad.y, s.rad.z, 0.0f);
    b.rng[k] = s.rs;
    b.depth[k] = s.depth;
    b.id[k] = s.id;
    if (cache) {
        b.spread[k] = s.sp;
        b.pflags[k] = s.fl;
    }
}

__device__ __forceinline__ int warp_append(int *counter, bool pred) {
    const unsigned m = __ballot_sync(~0u, pred);
    if (m == 0u) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(~0u, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

__device__ __forceinline__ void warp_add_u64(unsigned long long *dst, unsigned v) {
    unsigned long long x = v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(~0u, x, o);
    if ((threadIdx.x & 31) == 0 && x) atomicAdd(dst, x);
}

__device__ __forceinline__ float3 env_or_bg_ref(const DevScene &s, float3 d) {
    return s.env ? env_lookup_ref(s, d) : f3(1.0f, 1.0f, 1.0f);
}

// Generate1stRay (struct_Camera.cuh:38-45); jx, jy shift the pixel position.
__device__ __forceinline__ float3 primary_dir(const kgk_camera &c, int W, int H, float X, float Y) {
    const float3 cd = f3(c.CamDir.x, c.CamDir.y, c.CamDir.z);
    const float3 sx = f3(c.ScreenXDir.x, c.ScreenXDir.y, c.ScreenXDir.z);
    const float3 sy = f3(c.ScreenYDir.x, c.ScreenYDir.y, c.ScreenYDir.z);
    float3 r = cd * c.CamToScreenDist + (sx * (X - W / 2.0f)) * c.PixelSize + (sy * (H / 2.0f - Y)) * c.PixelSize;
    return normalize3(r);
}

// ---------------------------------------------------------------------------
// Primary ray of wave path i (pixel i % npx, sample sample_base + i / npx):
// origin, direction and the path's rng state.
__device__ __forceinline__ void primary_ray(const Params &P, int i, float3 &dir_out, unsigned long long &s_out) {
    const int px = i % P.npx;
    const int smp = P.sample_base + i / P.npx;
    const int X = px % P.W, Y = px / P.W;
    unsigned long long s;
    float3 dir;
    if (P.estimator == KGK_ESTIMATOR_COMPAT) {
        // render.cuh:29 seeding; pixel 0 divides by zero there, its terms are 0 here
        const int pos = px;
        const int m1 = (int)((unsigned)142857u * (unsigned)pos);
        const long long q = pos > 0 ? 998244353 / pos : 0;
        const long long r = pos > 0 ? 1000000007 % pos : 0;
        s = P.seeds[px] + (unsigned long long)(long long)m1 + (unsigned long long)q + (unsigned long long)r;
        dir = primary_dir(P.cam, P.W, P.H, (float)X, (float)Y);
    } else {
        s = splitmix64(P.seed ^ splitmix64(((unsigned long long)P.frame_index << 40) ^
                                           ((unsigned long long)smp << 26) ^ (unsigned long long)px));
        if (s == 0ull) s = 1ull;
        const float jx = rnd_u(s) - 0.5f, jy = rnd_u(s) - 0.5f;
        dir = primary_dir(P.cam, P.W, P.H, (float)X + jx, (float)Y + jy);
    }
    dir_out = dir;
    s_out = s;
}

// The path that buffer slot i of a wave starts: slots run over 8 x 4-pixel
// tiles (tiles in row order, pixels in row order inside a tile), so that a
// warp's 32 primary rays - and the shadow and secondary rays that follow
// them - leave one compact patch of the image.  The path index itself keeps
// its meaning (pixel = index % npx, sample = index / npx); images whose sides
// are not multiples of 8 and 4 keep scanline order.
__device__ __forceinline__ int tiled_path(const Params &P, int i) {
    if ((P.W & 7) || (P.H & 3)) return i;
    const int q = i % P.npx, t = q >> 5, w = q & 31, tw = P.W >> 3;
    return (i - q) + ((t / tw) * 4 + (w >> 3)) * P.W + (t % tw) * 8 + (w & 7);
}

__global__ void k_raygen(Params P) {
    const int n = P.npx * P.spp_wave;
    for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < n; slot += gridDim.x * blockDim.x) {
        const int i = slot, id = tiled_path(P, slot);
        float3 dir;
        unsigned long long s;
        primary_ray(P, id, dir, s);
        const PathBuf &b = P.cur;
        b.o[i] = make_float4(P.cam.CamOrg.x, P.cam.CamOrg.y, P.cam.CamOrg.z, 0.0f);
        b.d[i] = make_float4(dir.x, dir.y, dir.z, 0.0f);  // w: pdf of the sampled direction (0 = no MIS)
        b.thr[i] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        const float r0 = P.estimator == KGK_ESTIMATOR_COMPAT ? kSINF : 0.0f;  // RayTrace.cuh:14
        b.rad[i] = make_float4(r0, r0, r0, 0.0f);
        b.rng[i] = s;
        b.depth[i] = 0;
        b.id[i] = id;
        if (P.use_cache) {
            b.spread[i] = make_float2(0.0f, 0.0f);
            const bool train = P.train_stride > 0 && id < P.npx && (id % P.train_stride) == P.train_offset;
            b.pflags[i] = train ? 1 : 0;
        }
    }
}

// ---------------------------------------------------------------------------
// Closest hit of every live path (slots 0..n-1 of the current buffer; n from
// counter cnt_idx, or dense_n when cnt_idx < 0), written to hit[slot]; the
// slot goes to the miss, the Lambert or the Disney queue (the hit triangle's
// material class is in its BVH record, read by the traversal anyway), so
// shading warps are material-coherent.  Each warp gathers its finished slots
// in shared memory and appends them 32 at a time (one atomic, one coalesced
// store).
// Each warp keeps its lanes busy: when kRefill or more lanes have finished,
// they take the next rays (one atomic per warp).
struct QueueBatch {
    int *buf;       // this warp's 64 shared-memory entries
    int n = 0;      // entries held (warp-uniform, < 32 between calls)
    // Adds the lanes' slots where pred holds; writes out full batches of 32.
    __device__ __forceinline__ void add(bool pred, int slot, int *queue, int *counter) {
        const unsigned lane = threadIdx.x & 31u;
        const unsigned m = __ballot_sync(~0u, pred);
        if (pred) buf[n + __popc(m & ((1u << lane) - 1u))] = slot;
        n += __popc(m);
        __syncwarp();
        if (n >= 32) {
            int base = 0;
            if (lane == 0) base = atomicAdd(counter, 32);
            base = __shfl_sync(~0u, base, 0);
            queue[base + lane] = buf[lane];
            __syncwarp();
            if ((int)lane < n - 32) buf[lane] = buf[32 + lane];
            n -= 32;
            __syncwarp();
        }
    }
    // Writes out what is left.
    __device__ __forceinline__ void flush(int *queue, int *counter) {
        const unsigned lane = threadIdx.x & 31u;
        if (n == 0) return;
        int base = 0;
        if (lane == 0) base = atomicAdd(counter, n);
        base = __shfl_sync(~0u, base, 0);
        if ((int)lane < n) queue[base + lane] = buf[lane];
        n = 0;
    }
};

template <bool kCount>
__global__ void __launch_bounds__(128, 8) k_extend(Params P, int cnt_idx, int dense_n, int *mq, int *lq, int *dq) {
    const int n = cnt_idx >= 0 ? P.cnt[cnt_idx] : dense_n;
    const DevScene &s = P.sc;
    int *fetch = &P.cnt[kFE];
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt = (1u << lane) - 1u;
    __shared__ int s_q[3][4][64];  // per warp: miss, Lambert, Disney batches (blocks of 128 threads)
    QueueBatch mb, lb, db;
    mb.buf = s_q[0][threadIdx.x >> 5];
    lb.buf = s_q[1][threadIdx.x >> 5];
    db.buf = s_q[2][threadIdx.x >> 5];
    bool active = false, exhausted = false;
    int p = 0;
    unsigned rays = 0;
    RayPre r;
    Trav c;
    TravStack stk;
    TravStats st{0, 0, 0};
    while (true) {
        const unsigned idle = __ballot_sync(~0u, !active);
        if (!exhausted && __popc(idle) >= kRefill) {
            int base = 0;
            if (lane == 0) base = atomicAdd(fetch, __popc(idle));
            base = __shfl_sync(~0u, base, 0);
            if (base + __popc(idle) >= n) exhausted = true;
            if (!active) {
                const int i = base + __popc(idle & lt);
                if (i < n) {
                    p = i;
                    const float4 o = P.cur.o[p], d = P.cur.d[p];
                    r = make_ray(f3(o), f3(d));
                    trav_init(c, kBigT);
                    active = true;
                }
            }
        }
        if (!__any_sync(~0u, active)) break;
        int cls = -1;
        if (active && trav_step<kCount>(s.nodes, (unsigned)s.n_nodes, s.tri_rec, (unsigned)s.n_tris, r, c, stk,
                                        false, st)) {
            active = false;
            ++rays;
            cls = c.hit_slot < 0 ? 0 : 1 + (c.hit_slot & 1);
            P.hit[p] = c.hit_slot < 0 ? make_float4(kBigT, 0.0f, 0.0f, __int_as_float(-1))
                                      : make_float4(c.best_t, c.bu, c.bv, __int_as_float(c.best_id));
        }
        if (__any_sync(~0u, cls >= 0)) {
            mb.add(cls == 0, p, mq, &P.cnt[kMQ]);
            lb.add(cls == 1, p, lq, &P.cnt[kLQ]);
            db.add(cls == 2, p, dq, &P.cnt[kDQ]);
        }
    }
    mb.flush(mq, &P.cnt[kMQ]);
    lb.flush(lq, &P.cnt[kLQ]);
    db.flush(dq, &P.cnt[kDQ]);
    warp_add_u64(&P.stats[kRaysC], rays);
    if (kCount) {
        warp_add_u64(&P.stats[kNodes], st.nodes);
        warp_add_u64(&P.stats[kTris], st.tris);
    }
    warp_add_u64(&P.stats[kOverflow], st.overflow);
}

// ---------------------------------------------------------------------------
// Surface interaction (shared by both estimators)
// ---------------------------------------------------------------------------
struct Surface {
    float3 pos, ng, ns, n;  // n = shading normal flipped to face the ray
    float t;
    kgk_material m;
    int mat_id;
};

__device__ __forceinline__ Surface load_surface(const DevScene &s, int id, float4 h, float3 o, float3 d) {
    Surface S;
    const float3 v0 = f3(__ldg(&s.verts[3 * id])), v1 = f3(__ldg(&s.verts[3 * id + 1])),
                 v2 = f3(__ldg(&s.verts[3 * id + 2]));
    const float4 a0 = __ldg(&s.attr[4 * id]), a1 = __ldg(&s.attr[4 * id + 1]), a2 = __ldg(&s.attr[4 * id + 2]),
                 a3 = __ldg(&s.attr[4 * id + 3]);
    const float3 c = cross3(v1 - v0, v2 - v0);
    const float3 n0 = f3(a0), n1 = f3(a1), n2 = f3(a2);
    // Triangle::intersectTest (struct_Triangle.cuh:33-39, 62-76)
    S.ng = len3(c) == 0.0f ? normalize3(n0 + n1 + n2) : normalize3(c);
    const float b1 = h.y, b2 = h.z, b0 = 1.0f - b1 - b2;
    const unsigned bits = __float_as_uint(a3.w);
    S.ns = (bits & 0x80000000u) ? normalize3(n1 * b1 + n2 * b2 + n0 * b0) : S.ng;
    // u * v1_vt + v * v2_vt + (1 - u - v) * v0_vt (struct_Triangle.cuh:61),
    // rounded in the reference's order; k_tri_soa packs vt0 in a0.w / a1.w,
    // vt1 in a2.w / a3.x and vt2 in a3.y / a3.z
    const float w0 = __fsub_rn(__fsub_rn(1.0f, b1), b2);
    float uu = __fadd_rn(__fadd_rn(__fmul_rn(b1, a2.w), __fmul_rn(b2, a3.y)), __fmul_rn(w0, a0.w));
    float vv = __fadd_rn(__fadd_rn(__fmul_rn(b1, a3.x), __fmul_rn(b2, a3.z)), __fmul_rn(w0, a1.w));
    if (uu < 0.0f) uu += (float)((int)(-uu) + 1); else if (uu > 1.0f) uu -= (float)((int)uu);
    if (vv < 0.0f) vv += (float)((int)(-vv) + 1); else if (vv > 1.0f) vv -= (float)((int)vv);
    S.t = h.x;
    S.pos = o + d * h.x;
    S.mat_id = (int)(bits & 0x7fffffffu);
    S.m = s.mats[S.mat_id];
    if (S.m.TEXTURE_BASECOLOR_ID != -1) {
        const float3 tc = tex_fetch(s, S.m.TEXTURE_BASECOLOR_ID, uu, vv);
        S.m.diffuse.x = tc.x; S.m.diffuse.y = tc.y; S.m.diffuse.z = tc.z;
    }
    const float3 dif = f3(S.m.diffuse.x, S.m.diffuse.y, S.m.diffuse.z);
    if ((double)len3(dif) < 1e-5) {  // RayTrace.cuh:53-55
        S.m.diffuse.x = S.m.diffuse.y = S.m.diffuse.z = kSINF;
    }
    S.n = dot3(S.ns, d) > 0.0f ? -S.ns : S.ns;
    return S;
}

__device__ __forceinline__ float3 emission_of(const kgk_material &m) { return f3(m.emission.x, m.emission.y, m.emission.z); }
__device__ __forceinline__ float3 diffuse_of(const kgk_material &m) { return f3(m.diffuse.x, m.diffuse.y, m.diffuse.z); }

__device__ __forceinline__ void push_shadow(const Params &P, float4 *so, float4 *sd, float4 *sc, int cidx,
                                            bool pred, float3 org, float3 dir, float tmax, int light,
                                            float3 contrib, int target) {
    const int k = warp_append(&P.cnt[cidx], pred);
    if (pred) {
        so[k] = make_float4(org.x, org.y, org.z, tmax);
        sd[k] = make_float4(dir.x, dir.y, dir.z, __int_as_float(light));
        sc[k] = make_float4(contrib.x, contrib.y, contrib.z, __int_as_float(target));
    }
}

// Writes the G-buffer of a primary hit (RayTrace.cuh:66-82): albedo after the
// texture and the zero fix, emission, normal facing the camera, object id,
// material id, depth.  The reference's reprojection result is always
// (-1, -1) (struct_Camera.cuh:109-110); reprojection is done by SVGF itself.
__device__ __forceinline__ void write_gbuffer(const Params &P, int px, const Surface *S) {
    if (!S) {
        P.gb_pos[px] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        P.gb_nrm[px] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
        P.gb_alb[px] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
        P.gb_emi[px] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    P.gb_pos[px] = make_float4(S->pos.x, S->pos.y, S->pos.z, S->t);
    P.gb_alb[px] = make_float4(S->m.diffuse.x, S->m.diffuse.y, S->m.diffuse.z, __int_as_float(S->mat_id));
    P.gb_emi[px] = make_float4(S->m.emission.x, S->m.emission.y, S->m.emission.z, 1.0f);
}

// ---------------------------------------------------------------------------
// compat shade: RayTrace.cuh:37-106 for one vertex
// ---------------------------------------------------------------------------
// Result of one shading event: whether the path continues (its state is
// updated in place) and its shadow-ray records (face light: origin, direction,
// range, light id for the reference's closest-hit test or -1 for an occlusion
// test; environment: from spos), which the caller traces or queues.
struct ShadeOut {
    bool cont, f_pred, e_pred;
    float3 spos, f_org, f_dir, f_c, e_dir, e_c;
    float f_tmax;
    int f_light;
};

// A path that left the scene (either estimator): its G-buffer record when it
// is a first-sample camera ray, and the sky (or background) radiance it
// gathers - RayTrace.cuh:21-35 for the reference's estimator; with the
// environment's MIS weight against the sampled direction's pdf for the
// unbiased one.
template <int kEst>
__device__ __forceinline__ void shade_miss(const Params &P, float3 d, float prev_pdf, float3 T, float3 &rad,
                                           int depth, int path) {
    const DevScene &s = P.sc;
    const int px = path % P.npx;
    if (depth == 0 && P.write_gbuffer && path < P.npx) write_gbuffer(P, px, nullptr);
    if (kEst == KGK_ESTIMATOR_COMPAT) {
        rad += T * env_or_bg_ref(s, d);
    } else if (s.env) {
        const float3 Le = env_lookup_u(s, d);
        float wgt = 1.0f;
        if (prev_pdf > 0.0f) {
            const float pe = env_pdf_u(s, d);
            wgt = prev_pdf / (prev_pdf + pe);
        }
        rad += T * Le * wgt;
    } else {
        rad += T;  // background (1,1,1), no light sampling for it
    }
}

// One shading event of path ps (hit h) in the reference's estimator (see
// shade_unbiased_core).
__device__ __forceinline__ void shade_compat_core(const Params &P, PathState &ps, float4 h, ShadeOut &out) {
    const DevScene &s = P.sc;
    bool cont = false;
    bool f_pred = false, e_pred = false;
    float3 f_org, f_dir, f_c, e_dir, e_c;
    float f_tmax = 0.0f;
    int f_light = -1;
    float3 npos, ndir, T;
    unsigned long long rs = 0;
    {
        const float3 o = ps.o, d = ps.d;
        T = ps.T;
        float3 rad = ps.rad;
        rs = ps.rs;
        const int depth = ps.depth;
        const int id = __float_as_int(h.w);
        const int px = ps.id % P.npx;
        const bool first_sample = ps.id < P.npx;
        if (id < 0) {
            shade_miss<KGK_ESTIMATOR_COMPAT>(P, d, 0.0f, T, rad, depth, ps.id);
        } else {
            Surface S = load_surface(s, id, h, o, d);
            const float3 n = S.n;
            if (depth == 0 && P.write_gbuffer && first_sample) {
                write_gbuffer(P, px, &S);
                P.gb_nrm[px] = make_float4(n.x, n.y, n.z, __int_as_float(id));
            }
            const DisneyParams dp = disney_params(S.m);
            const float3 dif = diffuse_of(S.m), emi = emission_of(S.m);
            // Russian roulette (2, 3)
            float prr = fmaxf(dif.x, fmaxf(dif.y, dif.z));
            if (prr == 0.0f) prr = kSINF;
            const float rnd = rnd_ref(rs, 0.0f, 1.0f);
            bool killed = false;
            if (depth > 3) prr /= (float)(depth * depth);
            if (depth > 2) {
                if (prr < rnd) {
                    rad += T * emi;
                    killed = true;
                }
            } else {
                prr = 1.0f;
            }
            if (!killed) {
                if (depth == 0) rad += T * emi;
                T = T / prr;
                const float3 wo = -d;
                // NEE, face lights (NextEventEstimation_FaceLight.cuh:47-120)
                if (len3(emi) == 0.0f && S.m.MATERIAL_TYPE_ID < 2 && s.n_tris > 0) {
                    const float R = rnd_ref(rs, 0.0f, 1.0f);
                    // g++ evaluates SamplePointOnTriangle's arguments right to left
                    const float r2 = rnd_ref(rs, 0.0f, 1.0f);
                    const float r1 = rnd_ref(rs, 0.0f, 1.0f);
                    // without face lights the reference samples Objects[-1]
                    // (undefined); this step then contributes nothing
                    if (!s.no_light) {
                        const int lid = lower_bound_f(s.light_cdf_ref, s.n_tris,
                                                      R * __ldg(&s.light_cdf_ref[s.n_tris - 1]));
                        const float3 L0 = f3(__ldg(&s.verts[3 * lid])), L1 = f3(__ldg(&s.verts[3 * lid + 1])),
                                     L2 = f3(__ldg(&s.verts[3 * lid + 2]));
                        float t1 = r1 / 2.0f, t2 = r2 / 2.0f;
                        const float off = t2 - t1;
                        if (off > 0.0f) t2 += off; else t1 -= off;
                        const float3 Pl = L0 * t1 + L1 * t2 + L2 * (1.0f - t1 - t2);
                        const float3 Ld = normalize3(Pl - S.pos);
                        const float dist = len3(Pl - S.pos);
                        if (dot3(Ld, n) > 0.0f) {
                            // the light's shading normal at the sample (smooth lights interpolate)
                            const float4 la0 = __ldg(&s.attr[4 * lid]), la1 = __ldg(&s.attr[4 * lid + 1]),
                                         la2 = __ldg(&s.attr[4 * lid + 2]), la3 = __ldg(&s.attr[4 * lid + 3]);
                            const float3 lc = cross3(L1 - L0, L2 - L0);
                            float3 lng = len3(lc) == 0.0f ? normalize3(f3(la0) + f3(la1) + f3(la2)) : normalize3(lc);
                            if (__float_as_uint(la3.w) & 0x80000000u)
                                lng = normalize3(f3(la1) * t2 + f3(la2) * (1.0f - t1 - t2) + f3(la0) * t1);
                            const float cos1 = fabsf(dot3(S.ns, Ld)), cos2 = fabsf(dot3(lng, -Ld));
                            const float G = cos1 * cos2 / (dist * dist);
                            const float ltot = __ldg(&s.light_cdf_ref[s.n_tris - 1]);
                            const float lprev = lid == 0 ? 0.0f : __ldg(&s.light_cdf_ref[lid - 1]);
                            const float larea = 0.5f * len3(lc);
                            const float pdf_nee = (lid == 0 ? __ldg(&s.light_cdf_ref[0]) / ltot
                                                            : (__ldg(&s.light_cdf_ref[lid]) - lprev) / ltot) *
                                                  (1.0f / larea);
                            float p_hdr = s.env ? env_pdf_ref(s, Ld) : 0.0f;
                            float3 bsdf;
                            float p_pt;
                            if (S.m.MATERIAL_TYPE_ID == 0) {
                                bsdf = dif / kPI;
                                p_pt = fmaxf(dot3(n, Ld), 0.0f) / kPI;
                            } else {
                                float3 u, v, w;
                                onb_ref(n, u, v, w);
                                bsdf = disney_eval(S.m, dp, Ld, wo, n, u, v, w);
                                p_pt = disney_pdf_ref(dp, wo, Ld, n, u, v, w);
                            }
                            p_pt *= G / fabsf(dot3(Ld, S.ns));
                            const float mis = pdf_nee / (p_pt + pdf_nee + p_hdr);
                            const kgk_material lm = s.mats[__float_as_uint(la3.w) & 0x7fffffffu];
                            const float3 c = ((bsdf * G) / pdf_nee) * emission_of(lm) * mis;
                            f_pred = true;
                            f_org = S.pos;
                            f_dir = Ld;
                            f_tmax = dist * 1.001f + 1e-4f;
                            f_light = lid;
                            f_c = T * c;
                        }
                    }
                }
                // NEE, environment (NextEventEstimation_HDR.cuh:4-58)
                if (s.env) {
                    const int npx = s.env_w * s.env_h;
                    const float R = rnd_ref(rs, 0.0f, 1.0f);
                    const float tot = __ldg(&s.env_cdf_ref[npx - 1]);
                    const int pix = lower_bound_f(s.env_cdf_ref, npx, R * tot);
                    float pdf = pix == 0 ? __ldg(&s.env_cdf_ref[0]) / tot
                                         : (__ldg(&s.env_cdf_ref[pix]) - __ldg(&s.env_cdf_ref[pix - 1])) / tot;
                    const float3 ed = env_index_to_dir_ref(s, pix, pdf);
                    if (dot3(ed, n) > 0.0f) {
                        const float3 Le = env_texel(s, pix);
                        float3 bsdf;
                        float p_pt;
                        if (S.m.MATERIAL_TYPE_ID == 0) {
                            bsdf = dif / kPI;
                            p_pt = fmaxf(dot3(n, ed), 0.0f) / kPI;
                        } else {
                            float3 u, v, w;
                            onb_ref(n, u, v, w);
                            bsdf = disney_eval(S.m, dp, ed, wo, n, u, v, w);
                            p_pt = disney_pdf_ref(dp, wo, ed, n, u, v, w);
                        }
                        const float mis = pdf / (p_pt + pdf);
                        const float3 c = (bsdf * (Le / pdf)) * dot3(n, ed) * mis;
                        e_pred = true;
                        e_dir = ed;
                        e_c = c * T;
                    }
                }
                float3 u, v, w;
                onb_ref(n, u, v, w);
                // NextEventEstimation_PathTracing.cuh: draws its direction, adds nothing
                if (S.m.MATERIAL_TYPE_ID == 0) (void)sample_cos_ref(rs, u, v, w);
                // SampleNextRay (sampling.cuh:28-64)
                float3 nd;
                if (S.m.MATERIAL_TYPE_ID == 0) {
                    nd = sample_cos_ref(rs, u, v, w);
                    T = dif * T;
                } else {
                    // sample_BXDF in its zero-initialised reading: Sum = {w0, w0, w1, w2, w3}
                    float R = rnd_ref(rs, 0.0f, 1.0f);
                    const float sum[5] = {dp.wt[0], dp.wt[0], dp.wt[1], dp.wt[2], dp.wt[3]};
                    R *= sum[4];
                    int lobe;
                    {
                        int ng = -1, ok = 4;
                        while (ok - ng > 1) {
                            const int mid = (ok + ng) / 2;
                            if (sum[mid] >= R) ok = mid; else ng = mid;
                        }
                        lobe = ok;
                    }
                    if (lobe <= 2) {
                        nd = sample_cos_ref(rs, u, v, w);
                    } else if (lobe == 3) {
                        const float R1 = rnd_ref(rs, 0.0001f, 0.9999f);
                        const float R2 = rnd_ref(rs, 0.0001f, 0.9999f);
                        nd = reflect_ref(d, gtr2_half(R1, R2, u, v, w, dp.ax, dp.ay));
                    } else {
                        const float R1 = rnd_ref(rs, 0.0001f, 0.9999f);
                        const float R2 = rnd_ref(rs, 0.0001f, 0.9999f);
                        nd = reflect_ref(d, gtr1_half(R1, R2, u, v, w, dp.ac, false));
                    }
                    const float3 b = disney_eval(S.m, dp, nd, wo, n, u, v, w);
                    const float pdf = disney_pdf_ref(dp, wo, nd, n, u, v, w);
                    T = T * ((b * fabsf(dot3(n, nd))) / pdf);
                }
                npos = S.pos;
                ndir = nd;
                cont = P.max_depth <= 0 || depth + 1 < P.max_depth;
            }
        }
        ps.rad = rad;
        if (cont) {
            ps.o = npos;
            ps.d = ndir;
            ps.pdf = 0.0f;
            ps.T = T;
            ps.depth = depth + 1;
        }
        ps.rs = rs;
        if (!cont) P.seeds[px] = rs;  // randSeeds[pos] = rand.seed (render.cuh:42)
    }
    out.cont = cont;
    out.f_pred = f_pred;
    out.e_pred = e_pred;
    out.spos = npos;
    out.f_org = f_org;
    out.f_dir = f_dir;
    out.f_c = f_c;
    out.e_dir = e_dir;
    out.e_c = e_c;
    out.f_tmax = f_tmax;
    out.f_light = f_light;
}

// ---------------------------------------------------------------------------
// unbiased shade
// ---------------------------------------------------------------------------
// Not inlined: the unbiased shader evaluates the BSDF at three call sites
// (face-light NEE, environment NEE, BSDF sample); one copy of the Disney
// code keeps the kernel inside the instruction cache.  The material is read
// from its global record (diffuse passed in: it may come from a texture);
// returns (f, pdf).
__device__ __noinline__ float4 bsdf_eval_pdf(const kgk_material *__restrict__ mg, float3 diffuse, float3 n,
                                             float3 wo, float3 wi) {
    if (mg->MATERIAL_TYPE_ID == 1) {
        kgk_material m = *mg;
        m.diffuse.x = diffuse.x;
        m.diffuse.y = diffuse.y;
        m.diffuse.z = diffuse.z;
        const DisneyParams dp = disney_params(m);
        float3 u, v, w;
        onb_ref(n, u, v, w);
        const float3 f = disney_eval<false>(m, dp, wi, wo, n, u, v, w);
        return make_float4(f.x, f.y, f.z, disney_pdf_unbiased(dp, wo, wi, n, u, v, w));
    }
    const float c = dot3(n, wi);
    const float3 f = c > 0.0f ? diffuse / kPI : f3(0.0f, 0.0f, 0.0f);
    return make_float4(f.x, f.y, f.z, fmaxf(c, 0.0f) / kPI);
}

// bsdf_eval_pdf for a material class known at compile time: kMat 1 = Lambert
// (inline), otherwise the out-of-line evaluation of either class.
template <int kMat>
__device__ __forceinline__ float4 bsdf_eval_pdf_k(const kgk_material *__restrict__ mg, float3 diffuse, float3 n,
                                                  float3 wo, float3 wi) {
    if (kMat == 1) {
        const float c = dot3(n, wi);
        const float3 f = c > 0.0f ? diffuse / kPI : f3(0.0f, 0.0f, 0.0f);
        return make_float4(f.x, f.y, f.z, fmaxf(c, 0.0f) / kPI);
    }
    return bsdf_eval_pdf(mg, diffuse, n, wo, wi);
}

// Writes a cache record for the surface point of a path: normalised position,
// shading normal, direction to the viewer, roughness, albedo, then T, the
// path id and the radiance gathered so far.
__device__ __forceinline__ void write_cache_record(const Params &P, float *rec, const Surface &S, float3 wo,
                                                   float3 T, int path, float3 rad) {
    const DevScene &s = P.sc;
    const float3 lo = f3(s.lo[0], s.lo[1], s.lo[2]), hi = f3(s.hi[0], s.hi[1], s.hi[2]);
    const float3 e = hi - lo;
    rec[0] = fminf(fmaxf((S.pos.x - lo.x) / fmaxf(e.x, 1e-20f), 0.0f), 1.0f);
    rec[1] = fminf(fmaxf((S.pos.y - lo.y) / fmaxf(e.y, 1e-20f), 0.0f), 1.0f);
    rec[2] = fminf(fmaxf((S.pos.z - lo.z) / fmaxf(e.z, 1e-20f), 0.0f), 1.0f);
    rec[3] = S.n.x; rec[4] = S.n.y; rec[5] = S.n.z;
    rec[6] = wo.x; rec[7] = wo.y; rec[8] = wo.z;
    rec[9] = S.m.MATERIAL_TYPE_ID == 1 ? S.m.roughness : 1.0f;
    rec[10] = S.m.diffuse.x; rec[11] = S.m.diffuse.y; rec[12] = S.m.diffuse.z;
    rec[13] = T.x; rec[14] = T.y; rec[15] = T.z;
    rec[16] = __int_as_float(path);
    rec[17] = rad.x; rec[18] = rad.y; rec[19] = rad.z;
}

// One unbiased shading event of path ps (hit h): emission, the cache
// decisions, Russian roulette, the two NEE samples (returned in `out` as
// shadow-ray records, not traced) and the BSDF sample (ps updated).
// kMat: the material class of every path shaded here (1 Lambert, 2 Disney;
// 0: read from the material).
template <bool kCache, int kMat = 0>
__device__ __forceinline__ void shade_unbiased_core(const Params &P, PathState &ps, float4 h, ShadeOut &out) {
    const DevScene &s = P.sc;
    bool cont = false, f_pred = false, e_pred = false;
    float3 spos = f3(0.0f, 0.0f, 0.0f), f_dir = spos, f_c = spos, e_dir = spos, e_c = spos;
    float f_tmax = 0.0f, npdf = 0.0f;
    float3 ndir = spos, T = spos;
    unsigned long long rs = 0;
    {
        const float3 o = ps.o, d = ps.d;
        const float prev_pdf = ps.pdf;  // 0: no MIS (camera ray)
        T = ps.T;
        float3 rad = ps.rad;
        rs = ps.rs;
        const int depth = ps.depth;
        const int id = __float_as_int(h.w);
        const int px = ps.id % P.npx;
        const bool first_sample = ps.id < P.npx;
        if (id < 0) {
            shade_miss<KGK_ESTIMATOR_UNBIASED>(P, d, prev_pdf, T, rad, depth, ps.id);
        } else {
            // The environment NEE sample, drawn ahead: its random numbers sit
            // at a fixed place in the path's stream (after the Russian
            // roulette draw at depth >= rr_start and the emitter sample's
            // three), so it is drawn here on a copy of the state and its
            // alias-table and texel loads overlap the surface's.  Used (and
            // the state moved past it) only where the sequential order
            // draws it.
            unsigned long long rs_env = rs;
            float pe_env = 0.0f;
            float3 le_env = f3(0.0f, 0.0f, 0.0f), ed_env = le_env;
            if (s.env) {
                if (depth >= P.rr_start) rs_env = xorshift64(rs_env);
                if (s.n_emit > 0) rs_env = xorshift64(xorshift64(xorshift64(rs_env)));
                ed_env = env_sample_u(s, rs_env, pe_env, le_env);
            }
            Surface S = load_surface(s, id, h, o, d);
            const float3 n = S.n, wo = -d;
            if (depth == 0 && P.write_gbuffer && first_sample) {
                write_gbuffer(P, px, &S);
                P.gb_nrm[px] = make_float4(n.x, n.y, n.z, __int_as_float(id));
            }
            const float3 emi = emission_of(S.m);
            if (emi.x > 0.0f || emi.y > 0.0f || emi.z > 0.0f) {
                float wgt = 1.0f;
                if (prev_pdf > 0.0f && s.n_emit > 0) {
                    const float cosl = fabsf(dot3(S.ng, d));
                    const float parea = len3(emi) / s.emit_total;
                    const float pl = cosl > 0.0f ? parea * S.t * S.t / cosl : 0.0f;
                    wgt = prev_pdf / (prev_pdf + pl);
                }
                rad += T * emi * wgt;
            }
            bool alive = true;
            bool to_cache = false;
            if (kCache && P.use_cache) {
                // path spread (sqrt-summed) against the primary footprint
                float2 sp = ps.sp;
                const float cosl = fmaxf(fabsf(dot3(S.ng, d)), 1e-4f);
                if (depth == 0) sp.y = S.t * S.t / (4.0f * kPI * cosl);
                else sp.x += sqrtf(S.t * S.t / (fmaxf(prev_pdf, 1e-8f) * cosl));
                ps.sp = sp;
                int fl = ps.fl;
                const bool wide = depth >= 1 && sp.x * sp.x > P.spread_c * sp.y;
                if (fl & 1) {
                    if (!(fl & 2)) {
                        if (wide) {  // training path: record the query vertex, keep going
                            const int k = atomicAdd(&P.cnt[kTN], 1);
                            if (k < P.tcap) write_cache_record(P, P.trec + (size_t)k * kQRec, S, -d, T, ps.id, rad);
                            fl |= 2;
                        }
                    } else {
                        fl += 256;
                        if ((fl >> 8) >= P.suffix_max) to_cache = true;  // suffix end: bootstrap from the cache
                    }
                    ps.fl = fl;
                } else if (wide) {
                    to_cache = true;
                }
            }
            if (to_cache) {
                const int k = atomicAdd(&P.cnt[kQN], 1);
                write_cache_record(P, P.qrec + (size_t)k * kQRec, S, -d, T, ps.id, rad);
                alive = false;
            }
            if (alive && depth >= P.rr_start) {
                const float q = fminf(maxc(T), 0.95f);
                if (rnd_u(rs) >= q) alive = false;
                else T = T / q;
            }
            if (alive) {
                const DisneyParams dp = disney_params(S.m);
                spos = S.pos;
                // NEE: one emitter sample
                if (s.n_emit > 0) {
                    const float r0 = rnd_u(rs), r1 = rnd_u(rs), r2 = rnd_u(rs);
                    const int k = cdf_search(s.emit_cdf, s.n_emit, r0);
                    const int lid = __ldg(&s.emit_ids[min(k, s.n_emit - 1)]);
                    const float3 L0 = f3(__ldg(&s.verts[3 * lid])), L1 = f3(__ldg(&s.verts[3 * lid + 1])),
                                 L2 = f3(__ldg(&s.verts[3 * lid + 2]));
                    const float su = sqrtf(r1);
                    const float3 Pl = L0 * (1.0f - su) + L1 * (r2 * su) + L2 * (su - r2 * su);
                    float3 Ld = Pl - S.pos;
                    const float dist = len3(Ld);
                    Ld = Ld / dist;
                    const float3 lc = cross3(L1 - L0, L2 - L0);
                    const float cosl = fabsf(dot3(normalize3(lc), Ld));
                    const float coss = dot3(n, Ld);
                    if (coss > 0.0f && cosl > 0.0f && dist > 0.0f) {
                        const unsigned lb = __float_as_uint(__ldg(&s.attr[4 * lid + 3].w));
                        const float3 Le = emission_of(s.mats[lb & 0x7fffffffu]);
                        const float parea = len3(Le) / s.emit_total;
                        const float pl = parea * dist * dist / cosl;
                        const float4 fp = bsdf_eval_pdf_k<kMat>(&s.mats[S.mat_id], diffuse_of(S.m), n, wo, Ld);
                        const float3 f = f3(fp);
                        const float pb = fp.w;
                        const float wgt = pl / (pl + pb);
                        f_c = T * f * Le * (coss * wgt / pl);
                        f_pred = f_c.x > 0.0f || f_c.y > 0.0f || f_c.z > 0.0f;
                        f_dir = Ld;
                        f_tmax = dist * (1.0f - 1e-4f);
                    }
                }
                // NEE: one environment sample (drawn ahead)
                if (s.env) {
                    const float pe = pe_env;
                    const float3 Le = le_env, ed = ed_env;
                    rs = rs_env;
                    const float coss = dot3(n, ed);
                    if (coss > 0.0f && pe > 0.0f) {
                        const float4 fp = bsdf_eval_pdf_k<kMat>(&s.mats[S.mat_id], diffuse_of(S.m), n, wo, ed);
                        const float3 f = f3(fp);
                        const float pb = fp.w;
                        const float wgt = pe / (pe + pb);
                        e_c = T * f * Le * (coss * wgt / pe);
                        e_pred = e_c.x > 0.0f || e_c.y > 0.0f || e_c.z > 0.0f;
                        e_dir = ed;
                    }
                }
                // BSDF sample
                if (P.max_depth <= 0 || depth + 1 < P.max_depth) {
                    float3 u, v, w;
                    onb_ref(n, u, v, w);
                    float3 nd;
                    if (kMat == 2 || (kMat == 0 && S.m.MATERIAL_TYPE_ID == 1)) {
                        const float sw = dp.wt[0] + dp.wt[1] + dp.wt[2] + dp.wt[3] + dp.wt[4];
                        const float rl = rnd_u(rs) * sw, r1 = rnd_u(rs), r2 = rnd_u(rs);
                        const float c3 = dp.wt[0] + dp.wt[1] + dp.wt[2];
                        if (rl < c3) nd = sample_cos_u(r1, r2, u, v, w);
                        else if (rl < c3 + dp.wt[3])
                            nd = reflect_ref(d, gtr2_half(fminf(r1, 0.99999f), fminf(r2, 0.99999f), u, v, w, dp.ax, dp.ay));
                        else
                            nd = reflect_ref(d, gtr1_half(r1, r2, u, v, w, dp.ac, true));
                    } else {
                        const float r1 = rnd_u(rs), r2 = rnd_u(rs);
                        nd = sample_cos_u(r1, r2, u, v, w);
                    }
                    const float4 fp = bsdf_eval_pdf_k<kMat>(&s.mats[S.mat_id], diffuse_of(S.m), n, wo, nd);
                    const float3 f = f3(fp);
                    const float pb = fp.w;
                    const float c = dot3(n, nd);
                    if (pb > 0.0f && c > 0.0f) {
                        T = T * f * (c / pb);
                        if (T.x > 0.0f || T.y > 0.0f || T.z > 0.0f) {
                            cont = true;
                            ndir = nd;
                            npdf = pb;
                        }
                    }
                }
            }
        }
        ps.rad = rad;
        if (cont) {
            ps.o = spos;
            ps.d = ndir;
            ps.pdf = npdf;
            ps.T = T;
            ps.depth = depth + 1;
        }
        ps.rs = rs;
    }
    out.cont = cont;
    out.f_pred = f_pred;
    out.e_pred = e_pred;
    out.spos = spos;
    out.f_dir = f_dir;
    out.f_c = f_c;
    out.e_dir = e_dir;
    out.e_c = e_c;
    out.f_tmax = f_tmax;
    out.f_org = spos;
    out.f_light = -1;
}

// Shades the live paths of the current buffer with the hits k_extend wrote:
// first the miss queue (shade_miss: the sky lookup, then the path ends), then
// the Lambert and the Disney queues (the surface shading, on warps of one
// material class).
// Continuing paths move to the next buffer (counter next_cnt), finished ones
// leave their radiance in fin[id].  A shadow record names where its
// contribution goes: the path's slot in the next buffer (>= 0) or -(id + 1)
// for fin.
// kPart: 0 = all three queues in one launch; 1, 2, 3 = the miss, Lambert or
// Disney queue alone, each launch compiled for its class only (a smaller
// kernel: the one-launch form spends its time fetching instructions).
template <int kEst, bool kCache, int kPart = 0>
__global__ void __launch_bounds__(128) k_shade(Params P, const int *__restrict__ mq, const int *__restrict__ lq,
                                               const int *__restrict__ dq, int next_cnt, float4 *so0, float4 *sd0,
                                               float4 *sc0, float4 *so1, float4 *sd1, float4 *sc1) {
    const int nm = P.cnt[kMQ], nl = P.cnt[kLQ], nd = P.cnt[kDQ];
    // this launch's range of the list [misses, Lambert, Disney]
    const int lo = kPart == 2 ? nm : kPart == 3 ? nm + nl : 0;
    const int n = kPart == 1 ? nm : kPart == 2 ? nm + nl : nm + nl + nd;
    const bool cache = kCache && P.use_cache;
    for (int base = lo + blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const int j = base + threadIdx.x;
        if (kPart <= 1 && j < nm) {  // a miss: the path ends here
            const int i = mq[j];
            const PathBuf &b = P.cur;
            const float4 d4 = b.d[i];
            float3 rad = f3(b.rad[i]);
            const int path = b.id[i], depth = b.depth[i];
            shade_miss<kEst>(P, f3(d4), d4.w, f3(b.thr[i]), rad, depth, path);
            P.fin[path] = make_float4(rad.x, rad.y, rad.z, 0.0f);
            if (kEst == KGK_ESTIMATOR_COMPAT) P.seeds[path % P.npx] = b.rng[i];  // render.cuh:42
        }
        if (kPart == 1) continue;
        if (base + (int)blockDim.x <= nm) continue;  // the whole block was misses
        const bool go = j >= nm && j < n;
        PathState ps;
        ps.id = 0;
        ShadeOut o{};
        if (go) {
            const int jh = j - nm;
            const int i = jh < nl ? lq[jh] : dq[jh - nl];
            ps = load_path(P.cur, i, cache);
            if (kEst == KGK_ESTIMATOR_COMPAT) shade_compat_core(P, ps, P.hit[i], o);
            else shade_unbiased_core<kCache, kPart == 2 ? 1 : kPart == 3 ? 2 : 0>(P, ps, P.hit[i], o);
        }
        const int k = warp_append(&P.cnt[next_cnt], o.cont);
        if (o.cont) store_path(P.nxt, k, ps, cache);
        else if (go) P.fin[ps.id] = make_float4(ps.rad.x, ps.rad.y, ps.rad.z, 0.0f);
        const int target = o.cont ? k : -(ps.id + 1);
        push_shadow(P, so0, sd0, sc0, kSH0, o.f_pred, o.f_org, o.f_dir, o.f_tmax, o.f_light, o.f_c, target);
        push_shadow(P, so1, sd1, sc1, kSH1, o.e_pred, o.spos, o.e_dir, kBigT, -1, o.e_c, target);
    }
}

// The tail of a wave: once few paths are alive (or the whole wave is small),
// each thread carries one path of the current buffer (slots 0..n-1, n from
// counter cnt_idx, or dense_n when cnt_idx < 0) through all of its remaining
// bounces in registers - closest hit, shading, then its face-light and
// environment shadow rays in that order (the order of the wavefront's passes,
// so the radiance sums are the same) - instead of four kernel launches per
// bounce that each wait for their slowest ray.  A path runs at most `bounces`
// more bounces, the wavefront's limit.
// One deferred shadow record: slot (path i, bounce k, kind j) and its id in
// the list (warp-aggregated append; the list order does not matter).
__device__ __forceinline__ void defer_shadow(const Params &P, int i, int k, int j, float3 org, float3 dir,
                                             float tmax, float3 c) {
    const size_t slot = ((size_t)i * kDeferBounces + k) * 2 + j;
    P.td_o[slot] = make_float4(org.x, org.y, org.z, tmax);
    P.td_d[slot] = make_float4(dir.x, dir.y, dir.z, 0.0f);
    P.td_c[slot] = make_float4(c.x, c.y, c.z, 0.0f);
    cg::coalesced_group g = cg::coalesced_threads();
    int base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(&P.cnt[kTD], (int)g.size());
    base = g.shfl(base, 0);
    P.td_list[base + (int)g.thread_rank()] = (int)slot;
}

// Bounce k of tail path i in registers: closest hit, shading, then its
// face-light and environment shadow rays in that order (the order of the
// wavefront's passes, so the radiance sums are the same); with `defer`, the
// shadow rays of its first kDeferBounces bounces go to slots of tail path i
// instead, and bit 2k + j of dmask records record (bounce k, kind j).
// Returns whether the path continues.
template <int kEst, bool kCache>
__device__ __forceinline__ bool tail_bounce(const Params &P, PathState &ps, int i, int k, bool defer,
                                            unsigned &dmask, unsigned &rays_c, unsigned &rays_s,
                                            unsigned &overflow) {
    const DevScene &s = P.sc;
    const RayPre r = make_ray(ps.o, ps.d);
    float bt = kBigT, u = 0.0f, v = 0.0f;
    int bid = 0x7fffffff;
    TravStats st{0, 0, 0};
    const int slot = trace_closest<false>(s.nodes, (unsigned)s.n_nodes, s.tri_rec, (unsigned)s.n_tris, r, bt,
                                          bid, u, v, st);
    const float4 h = slot < 0 ? make_float4(kBigT, 0.0f, 0.0f, __int_as_float(-1))
                              : make_float4(bt, u, v, __int_as_float(bid));
    ++rays_c;
    ShadeOut so{};
    if (kEst == KGK_ESTIMATOR_COMPAT) shade_compat_core(P, ps, h, so);
    else shade_unbiased_core<kCache>(P, ps, h, so);
    if (defer && k < kDeferBounces) {
        if (so.f_pred) {
            defer_shadow(P, i, k, 0, so.f_org, so.f_dir, so.f_tmax, so.f_c);
            dmask |= 1u << (2 * k);
        }
        if (so.e_pred) {
            defer_shadow(P, i, k, 1, so.spos, so.e_dir, kBigT, so.e_c);
            dmask |= 2u << (2 * k);
        }
        so.f_pred = so.e_pred = false;
    }
    if (so.f_pred) {
        const RayPre rs = make_ray(so.f_org, so.f_dir);
        bool vis;
        if (so.f_light >= 0) {  // the reference's test: the closest hit is the light
            float lt = so.f_tmax, lu, lv;
            int lid = 0x7fffffff;
            const int ls = trace_closest<false>(s.nodes, (unsigned)s.n_nodes, s.tri_rec, (unsigned)s.n_tris,
                                                rs, lt, lid, lu, lv, st);
            vis = ls >= 0 && lid == so.f_light;
        } else {
            vis = !trace_any<false>(s.nodes, (unsigned)s.n_nodes, s.tri_rec, (unsigned)s.n_tris, rs,
                                    so.f_tmax, st);
        }
        if (vis) ps.rad = ps.rad + so.f_c;
        ++rays_s;
    }
    if (so.e_pred) {
        const RayPre rs = make_ray(so.spos, so.e_dir);
        if (!trace_any<false>(s.nodes, (unsigned)s.n_nodes, s.tri_rec, (unsigned)s.n_tris, rs, kBigT, st))
            ps.rad = ps.rad + so.e_c;
        ++rays_s;
    }
    overflow += st.overflow;
    return so.cont;
}

// Each thread carries one path at a time through at most `bounces` more
// bounces; the grid is what fits on the GPU at once.
// Unbiased estimator: one loop iteration runs one bounce of every lane's
// path.  A lane whose path has ended stays idle until kTailRefill lanes of
// its warp are idle (or the paths run out); then the idle lanes take the next
// paths together (one atomic for the warp) and load them.  So a warp neither
// waits for the longest of its 32 paths (most tail paths of a frame end after
// one bounce there) nor pays a fetch's latency on every bounce.
// Compat estimator: a loop over each thread's whole path, a new path from
// the counter when it ends.  Its waves run entirely in the tail from the
// primary rays (long paths that Russian roulette ends, on small scenes),
// where the refill loop measured slower.
template <int kEst, bool kCache>
__global__ void __launch_bounds__(128) k_tail(Params P, int cnt_idx, int dense_n, int bounces) {
    const int n = cnt_idx >= 0 ? P.cnt[cnt_idx] : dense_n;
    const bool cache = kCache;
    const bool defer = kEst == KGK_ESTIMATOR_UNBIASED && P.td_o != nullptr && n <= kTailPaths;
    const unsigned lane = threadIdx.x & 31u;
    unsigned rays_c = 0, rays_s = 0, overflow = 0;
    if constexpr (kEst == KGK_ESTIMATOR_COMPAT) {
        for (int i = atomicAdd(&P.cnt[kTF], 1); i < n; i = atomicAdd(&P.cnt[kTF], 1)) {
            PathState ps = load_path(P.cur, i, cache);
            unsigned dmask = 0;
            for (int k = 0; k < bounces; ++k)
                if (!tail_bounce<kEst, kCache>(P, ps, i, k, false, dmask, rays_c, rays_s, overflow)) break;
            P.fin[ps.id] = make_float4(ps.rad.x, ps.rad.y, ps.rad.z, 0.0f);
        }
        warp_add_u64(&P.stats[kRaysC], rays_c);
        warp_add_u64(&P.stats[kRaysS], rays_s);
        warp_add_u64(&P.stats[kRaysT], rays_c);
        warp_add_u64(&P.stats[kOverflow], overflow);
        return;
    }
    PathState ps;
    int i = -1, k = 0;
    unsigned dmask = 0;
    bool exhausted = false;
    while (true) {
        const unsigned idle = __ballot_sync(~0u, i < 0);
        if (!exhausted && (__popc(idle) >= kTailRefill || idle == ~0u)) {
            int base = 0;
            if (lane == 0) base = atomicAdd(&P.cnt[kTF], __popc(idle));
            base = __shfl_sync(~0u, base, 0);
            if (base + __popc(idle) >= n) exhausted = true;
            if (i < 0) {
                const int j = base + __popc(idle & ((1u << lane) - 1u));
                if (j < n) {
                    i = j;
                    ps = load_path(P.cur, i, cache);
                    k = 0;
                    dmask = 0;
                }
            }
        }
        if (!__any_sync(~0u, i >= 0)) {
            if (exhausted) break;
            continue;
        }
        if (i >= 0) {
            const bool cont =
                k < bounces && tail_bounce<kEst, kCache>(P, ps, i, k, defer, dmask, rays_c, rays_s, overflow);
            if (!cont || ++k >= bounces) {
                P.fin[ps.id] = make_float4(ps.rad.x, ps.rad.y, ps.rad.z, 0.0f);
                if (defer) P.td_mask[i] = dmask;
                i = -1;
            }
        }
    }
    warp_add_u64(&P.stats[kRaysC], rays_c);
    warp_add_u64(&P.stats[kRaysS], rays_s);
    warp_add_u64(&P.stats[kRaysT], rays_c);
    warp_add_u64(&P.stats[kOverflow], overflow);
}

// Paths still live when the bounce limit ends the wavefront: their radiance
// so far is final.
__global__ void k_flush(Params P, int cnt_idx) {
    const int n = P.cnt[cnt_idx];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        P.fin[P.cur.id[i]] = P.cur.rad[i];
}

// The tail's deferred shadow rays (any-hit: nothing in (kTMin, range)), from
// the list of filled slots, lanes refilled like k_extend's; the visibility
// of slot s goes to td_vis[s].
__global__ void __launch_bounds__(128, 8) k_tail_shadow(Params P) {
    const int n = P.cnt[kTD];
    const DevScene &s = P.sc;
    int *fetch = &P.cnt[kTDF];
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt = (1u << lane) - 1u;
    bool active = false, exhausted = false;
    int slot = 0;
    unsigned rays = 0;
    RayPre r;
    Trav c;
    TravStack stk;
    TravStats st{0, 0, 0};
    while (true) {
        const unsigned idle = __ballot_sync(~0u, !active);
        if (!exhausted && __popc(idle) >= kRefill) {
            int base = 0;
            if (lane == 0) base = atomicAdd(fetch, __popc(idle));
            base = __shfl_sync(~0u, base, 0);
            if (base + __popc(idle) >= n) exhausted = true;
            if (!active) {
                const int i = base + __popc(idle & lt);
                if (i < n) {
                    slot = P.td_list[i];
                    const float4 o = P.td_o[slot], d = P.td_d[slot];
                    r = make_ray(f3(o), f3(d));
                    trav_init(c, o.w);
                    active = true;
                }
            }
        }
        if (!__any_sync(~0u, active)) break;
        if (active && trav_step<false, kNodesPerStepShadow>(s.nodes, (unsigned)s.n_nodes, s.tri_rec,
                                                            (unsigned)s.n_tris, r, c, stk, true, st)) {
            active = false;
            ++rays;
            P.td_vis[slot] = c.hit_slot < 0 ? 1 : 0;
        }
    }
    warp_add_u64(&P.stats[kRaysS], rays);
    warp_add_u64(&P.stats[kOverflow], st.overflow);
}

// Adds each tail path's visible deferred contributions to its radiance, in
// slot order (bounce by bounce, face light before environment): the same sum
// on every run.
__global__ void k_tail_resolve(Params P, int cnt_idx, int dense_n) {
    const int n = min(cnt_idx >= 0 ? P.cnt[cnt_idx] : dense_n, kTailPaths);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        unsigned m = P.td_mask[i];
        if (!m) continue;
        const int id = P.cur.id[i];
        float4 rad = P.fin[id];
        while (m) {
            const int b = __ffs(m) - 1;
            m &= m - 1u;
            const size_t slot = (size_t)i * kDeferBounces * 2 + b;
            if (P.td_vis[slot]) {
                const float4 cc = P.td_c[slot];
                rad.x += cc.x;
                rad.y += cc.y;
                rad.z += cc.z;
            }
        }
        P.fin[id] = rad;
    }
}

// ---------------------------------------------------------------------------
// Shadow rays of one queue: a face-light record (light id >= 0) is visible
// when the closest hit within its range is that light (the reference's test,
// NextEventEstimation_FaceLight.cuh:69-71); an environment record when nothing
// lies in (kTMin, range).  Visible records add their contribution to the
// path's radiance - in the next buffer, or in fin for a finished path (one
// record per path per queue, so no atomics).  Lanes are refilled like
// k_extend's.
__global__ void __launch_bounds__(128, 8) k_shadow(Params P, int cidx, int fidx, const float4 *__restrict__ so,
                                                const float4 *__restrict__ sd, const float4 *__restrict__ sc) {
    const int n = P.cnt[cidx];
    const DevScene &s = P.sc;
    int *fetch = &P.cnt[fidx];
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt = (1u << lane) - 1u;
    bool active = false, exhausted = false;
    int i = 0, light = -1;
    unsigned rays = 0;
    RayPre r;
    Trav c;
    TravStack stk;
    TravStats st{0, 0, 0};
    while (true) {
        const unsigned idle = __ballot_sync(~0u, !active);
        if (!exhausted && __popc(idle) >= kRefill) {
            int base = 0;
            if (lane == 0) base = atomicAdd(fetch, __popc(idle));
            base = __shfl_sync(~0u, base, 0);
            if (base + __popc(idle) >= n) exhausted = true;
            if (!active) {
                i = base + __popc(idle & lt);
                if (i < n) {
                    const float4 o = so[i], d = sd[i];
                    r = make_ray(f3(o), f3(d));
                    light = __float_as_int(d.w);
                    trav_init(c, o.w);
                    active = true;
                }
            }
        }
        if (!__any_sync(~0u, active)) break;
        if (active && trav_step<false, kNodesPerStepShadow>(s.nodes, (unsigned)s.n_nodes, s.tri_rec,
                                                            (unsigned)s.n_tris, r, c, stk, light < 0, st)) {
            active = false;
            ++rays;
            const bool vis = light >= 0 ? (c.hit_slot >= 0 && c.best_id == light) : c.hit_slot < 0;
            if (vis) {
                const float4 cc = sc[i];
                const int t = __float_as_int(cc.w);
                float4 *dst = t >= 0 ? P.nxt.rad + t : P.fin + (-t - 1);
                float4 rr = *dst;
                rr.x += cc.x;
                rr.y += cc.y;
                rr.z += cc.z;
                *dst = rr;
            }
        }
    }
    warp_add_u64(&P.stats[kRaysS], rays);
    warp_add_u64(&P.stats[kOverflow], st.overflow);
}

// Training targets: scattered radiance leaving each recorded query vertex,
// (radiance at the end of the path - radiance before the vertex) / T.
__global__ void k_cache_targets(const float *trec, const int *n_dev, int cap, const float4 *rad, float *tgt) {
    const int n = min(*n_dev, cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float *r = trec + (size_t)i * kQRec;
        const int path = __float_as_int(r[16]);
        const float4 fin = rad[path];
        const float f[3] = {fin.x, fin.y, fin.z};
        for (int c = 0; c < 3; ++c) tgt[3 * i + c] = (f[c] - r[17 + c]) / fmaxf(r[13 + c], 1e-8f);
    }
}

// Sums the wave's samples per pixel (fixed order) into the frame buffer and
// the FP64 accumulator.
__global__ void k_finish(Params P, float4 *frame, double *acc_sum, double *acc_sq, int accumulate, int first_wave) {
    for (int px = blockIdx.x * blockDim.x + threadIdx.x; px < P.npx; px += gridDim.x * blockDim.x) {
        float4 f = first_wave ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : frame[px];
        double s0 = 0, s1 = 0, s2 = 0, q0 = 0, q1 = 0, q2 = 0;
        for (int k = 0; k < P.spp_wave; ++k) {
            const float4 r = P.fin[k * P.npx + px];
            f.x += r.x;
            f.y += r.y;
            f.z += r.z;
            if (accumulate) {
                s0 += r.x; s1 += r.y; s2 += r.z;
                q0 += (double)r.x * r.x; q1 += (double)r.y * r.y; q2 += (double)r.z * r.z;
            }
        }
        frame[px] = f;
        if (accumulate) {
            acc_sum[3 * px] += s0; acc_sum[3 * px + 1] += s1; acc_sum[3 * px + 2] += s2;
            acc_sq[3 * px] += q0; acc_sq[3 * px + 1] += q1; acc_sq[3 * px + 2] += q2;
        }
    }
}

__global__ void k_output(const float4 *frame, int npx, float inv_spp, float4 *out) {
    for (int px = blockIdx.x * blockDim.x + threadIdx.x; px < npx; px += gridDim.x * blockDim.x) {
        const float4 f = frame[px];
        out[px] = make_float4(f.x * inv_spp, f.y * inv_spp, f.z * inv_spp, 1.0f);
    }
}

template <class T> kgk_status ensure(T **p, size_t n, const char *what) {
    dfree(*p);
    *p = nullptr;
    return dalloc(p, n, what);
}

kgk_status ensure_pixels(RenderState &R, int W, int H) {
    if (R.W == W && R.H == H && R.seeds) return KGK_OK;
    const size_t npx = (size_t)W * H;
    KGK_TRY(ensure(&R.seeds, npx, "per-pixel seeds"));
    KGK_CUDA(cudaMemset(R.seeds, 0, npx * sizeof(unsigned long long)));
    KGK_TRY(ensure(&R.frame, npx, "frame buffer"));
    KGK_TRY(ensure(&R.kept, npx, "frame buffer"));
    R.kept_valid = false;
    KGK_TRY(ensure(&R.gb_pos, npx, "G-buffer"));
    KGK_TRY(ensure(&R.gb_nrm, npx, "G-buffer"));
    KGK_TRY(ensure(&R.gb_alb, npx, "G-buffer"));
    KGK_TRY(ensure(&R.gb_emi, npx, "G-buffer"));
    R.W = W;
    R.H = H;
    return KGK_OK;
}

kgk_status ensure_wave(RenderState &R, int cap, bool cache) {
    if (R.cap >= cap && (!cache || R.qrec_cap >= cap)) return KGK_OK;
    if (cache && R.qrec_cap < cap) {
        for (int k = 0; k < 2; ++k) {
            KGK_TRY(ensure(&R.pb[k].spread, cap, "cache path state"));
            KGK_TRY(ensure(&R.pb[k].pflags, cap, "cache path state"));
        }
        KGK_TRY(ensure(&R.qrec, (size_t)cap * kQRec, "cache query records"));
        R.qrec_cap = cap;
    }
    if (R.cap >= cap) return KGK_OK;
    for (int k = 0; k < 2; ++k) {
        PathBuf &b = R.pb[k];
        KGK_TRY(ensure(&b.o, cap, "path state"));
        KGK_TRY(ensure(&b.d, cap, "path state"));
        KGK_TRY(ensure(&b.thr, cap, "path state"));
        KGK_TRY(ensure(&b.rad, cap, "path state"));
        KGK_TRY(ensure(&b.rng, cap, "path state"));
        KGK_TRY(ensure(&b.depth, cap, "path state"));
        KGK_TRY(ensure(&b.id, cap, "path state"));
    }
    KGK_TRY(ensure(&R.fin, cap, "path radiance"));
    KGK_TRY(ensure(&R.hit, cap, "path hits"));
    KGK_TRY(ensure(&R.mq, cap, "miss queue"));
    KGK_TRY(ensure(&R.lq, cap, "Lambert queue"));
    KGK_TRY(ensure(&R.dq, cap, "Disney queue"));
    for (int k = 0; k < 2; ++k) {
        KGK_TRY(ensure(&R.sh_o[k], cap, "shadow queue"));
        KGK_TRY(ensure(&R.sh_d[k], cap, "shadow queue"));
        KGK_TRY(ensure(&R.sh_c[k], cap, "shadow queue"));
    }
    R.cap = cap;
    return KGK_OK;
}

kgk_status ensure_tail_defer(RenderState &R) {
    if (R.td_o) return KGK_OK;
    KGK_TRY(ensure(&R.td_o, kDeferSlots, "deferred shadow rays"));
    KGK_TRY(ensure(&R.td_d, kDeferSlots, "deferred shadow rays"));
    KGK_TRY(ensure(&R.td_c, kDeferSlots, "deferred shadow rays"));
    KGK_TRY(ensure(&R.td_list, kDeferSlots, "deferred shadow rays"));
    KGK_TRY(ensure(&R.td_vis, kDeferSlots, "deferred shadow rays"));
    KGK_TRY(ensure(&R.td_mask, (size_t)kTailPaths, "deferred shadow rays"));
    return KGK_OK;
}

kgk_status ensure_train(RenderState &R, int tcap) {
    if (R.tcap >= tcap) return KGK_OK;
    KGK_TRY(ensure(&R.trec, (size_t)tcap * kQRec, "cache training records"));
    KGK_TRY(ensure(&R.ttgt, (size_t)tcap * 3, "cache training targets"));
    R.tcap = tcap;
    return KGK_OK;
}

}  // namespace

void render_state_free(kgk_scene *s) {
    RenderState *R = s->rs;
    if (!R) return;
    if (R->st2) cudaStreamDestroy(R->st2);
    if (R->shaded) cudaEventDestroy(R->shaded);
    if (R->shadowed) cudaEventDestroy(R->shadowed);
    void *ptrs[] = {R->seeds, R->frame, R->kept, R->acc_sum, R->acc_sq, R->gb_pos, R->gb_nrm, R->gb_alb, R->gb_emi,
                    R->fin, R->hit, R->mq, R->lq, R->dq, R->sh_o[0], R->sh_o[1], R->sh_d[0], R->sh_d[1], R->sh_c[0],
                    R->sh_c[1], R->cnt, R->stats, R->qrec, R->trec, R->ttgt, R->td_o, R->td_d, R->td_c,
                    R->td_list, R->td_mask, R->td_vis};
    for (void *p : ptrs) dfree(p);
    for (PathBuf &b : R->pb) {
        void *bp[] = {b.o, b.d, b.thr, b.rad, b.rng, b.depth, b.id, b.spread, b.pflags};
        for (void *p : bp) dfree(p);
    }
    delete R;
    s->rs = nullptr;
}

RenderState *render_state(kgk_scene *s) {
    if (!s->rs) s->rs = new RenderState();
    return s->rs;
}

bool render_kept_frame(kgk_scene *s, int *W, int *H, const float4 **frame) {
    RenderState *R = s->rs;
    if (!R || !R->kept_valid) return false;
    *W = R->W;
    *H = R->H;
    *frame = R->kept;
    return true;
}

bool svgf_gbuffer(kgk_scene *s, int *W, int *H, const float4 **pos, const float4 **nrm, const float4 **alb,
                  const float4 **emi, kgk_camera *cam) {
    RenderState *R = s->rs;
    if (!R || !R->gbuffer_valid) return false;
    *W = R->W;
    *H = R->H;
    *pos = R->gb_pos;
    *nrm = R->gb_nrm;
    *alb = R->gb_alb;
    *emi = R->gb_emi;
    *cam = R->gbuffer_cam;
    return true;
}

}  // namespace kgk

using namespace kgk;

extern "C" {

kgk_status kgk_render(kgk_scene *s, const kgk_camera *cam, const kgk_camera *prev_cam,
                      const kgk_render_config *cfg, kgk_vec *out, kgk_stats *stats) {
    (void)prev_cam;
    if (!s || !cam || !cfg) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_render: NULL argument");
    if (!s->built) return fail(KGK_ERR_NOT_BUILT, "kgk_render: call kgk_build_bvh first");
    if (cfg->width <= 0 || cfg->height <= 0 || (long long)cfg->width * cfg->height > (1LL << 26))
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_render: image size out of range");
    if (cfg->spp <= 0) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_render: spp must be positive");
    if (cfg->estimator != KGK_ESTIMATOR_COMPAT && cfg->estimator != KGK_ESTIMATOR_UNBIASED)
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_render: unknown estimator");
    if (cfg->use_cache && cfg->estimator != KGK_ESTIMATOR_UNBIASED)
        return fail(KGK_ERR_UNSUPPORTED, "kgk_render: the radiance cache works with the unbiased estimator");
    if (cfg->use_cache && (!s->nrc || !s->nrc->ready))
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_render: use_cache needs kgk_nrc_init");
    KGK_CUDA(cudaSetDevice(s->device));
    RenderState &R = *render_state(s);
    // A render that returned early with an error may have left its last shadow
    // passes running on the second stream; everything this call queues on the
    // scene's stream (counter resets first) waits for them.
    if (R.shadowed) KGK_CUDA(cudaStreamWaitEvent(s->stream, R.shadowed, 0));
    const int W = cfg->width, H = cfg->height, npx = W * H;
    KGK_TRY(ensure_pixels(R, W, H));
    if (cfg->estimator == KGK_ESTIMATOR_COMPAT && cfg->frame_index == 0)
        KGK_CUDA(cudaMemsetAsync(R.seeds, 0, (size_t)npx * sizeof(unsigned long long), s->stream));
    // samples per wave: compat chains the per-pixel seeds, one sample per wave
    int spw = 1;
    if (cfg->estimator == KGK_ESTIMATOR_UNBIASED) {
        // Default: as many paths in flight as fit in half of the free device
        // memory, up to 2^27 (a 1080p frame at 64 spp in one wave, ~28 GB of
        // path state): each bounce's last, latency-bound rays then overlap
        // with the bulk of the frame instead of ending every small wave.
        int target = cfg->wave_paths;
        if (target <= 0) {
            size_t free_b = 0, total_b = 0;
            KGK_CUDA(cudaMemGetInfo(&free_b, &total_b));
            const size_t per_path = kPathStateBytes + (cfg->use_cache ? kCachePathBytes : 0);
            const size_t fit = (free_b / 2 + R.cap_bytes_held()) / per_path;
            target = (int)std::min<size_t>((size_t)1 << 27, std::max<size_t>(fit, (size_t)npx));
        }
        spw = std::max(1, std::min(cfg->spp, target / std::max(npx, 1)));
    }
    KGK_TRY(ensure_wave(R, npx * spw, cfg->use_cache != 0));
    if (!R.cnt) KGK_TRY(dalloc(&R.cnt, kNCnt, "counters"));
    if (!R.stats) KGK_TRY(dalloc(&R.stats, kNStat, "counters"));
    if (cfg->accumulate) {
        if (!R.acc_sum || R.acc_W != W || R.acc_H != H)
            return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_render: accumulate needs kgk_accum_reset for this size");
    }
    if (!R.sms) {
        cudaDeviceProp prop;
        KGK_CUDA(cudaGetDeviceProperties(&prop, s->device));
        R.sms = prop.multiProcessorCount;
    }
    cudaStream_t st = s->stream;
    KGK_CUDA(cudaMemsetAsync(R.stats, 0, kNStat * sizeof(unsigned long long), st));
    Params P;
    memset(&P, 0, sizeof P);
    P.sc = s->dev;
    // whether shading can write face-light shadow records at all (the compat
    // estimator samples the reference's light CDF, the unbiased one the
    // emitter list); without, the face-light shadow pass is not launched
    const bool face_lights = cfg->estimator == KGK_ESTIMATOR_COMPAT ? !s->dev.no_light : s->dev.n_emit > 0;
    P.sc.tex_filter = cfg->texture_filter == 1 ? 1 : 0;
    P.cam = *cam;
    P.W = W;
    P.H = H;
    P.npx = npx;
    P.estimator = cfg->estimator;
    P.max_depth = cfg->max_depth;
    P.rr_start = cfg->rr_start_depth;
    P.write_gbuffer = cfg->write_gbuffer;
    P.count_work = cfg->count_work;
    P.seed = cfg->seed;
    P.frame_index = cfg->frame_index;
    P.cur = R.pb[0];
    P.nxt = R.pb[1];
    P.fin = R.fin;
    P.hit = R.hit;
    P.seeds = R.seeds;
    P.gb_pos = R.gb_pos; P.gb_nrm = R.gb_nrm; P.gb_alb = R.gb_alb; P.gb_emi = R.gb_emi;
    P.cnt = R.cnt;
    P.stats = R.stats;
    P.use_cache = cfg->use_cache ? 1 : 0;
    P.td_o = P.td_d = P.td_c = nullptr;
    P.td_list = nullptr;
    P.td_mask = nullptr;
    P.td_vis = nullptr;
    if (cfg->estimator != KGK_ESTIMATOR_COMPAT && !P.use_cache) {
        KGK_TRY(ensure_tail_defer(R));
        P.td_o = R.td_o;
        P.td_d = R.td_d;
        P.td_c = R.td_c;
        P.td_list = R.td_list;
        P.td_mask = R.td_mask;
        P.td_vis = R.td_vis;
    }
    if (P.use_cache) {
        const kgk_nrc_config &nc = s->nrc->cfg;
        KGK_TRY(ensure_train(R, nc.train_paths));
        P.qrec = R.qrec;
        P.trec = R.trec;
        P.tcap = R.tcap;
        P.train_stride = std::max(1, npx / std::max(nc.train_paths, 1));
        P.train_offset = (int)(((unsigned)cfg->frame_index * 2654435761u) % (unsigned)P.train_stride);
        P.suffix_max = nc.train_suffix_max;
        P.spread_c = nc.spread_c;
    }
    const int grid = R.sms * 8;   // persistent grid-stride launches, 128 threads per block
    if (!R.st2) {
        KGK_CUDA(cudaStreamCreateWithFlags(&R.st2, cudaStreamNonBlocking));
        KGK_CUDA(cudaEventCreateWithFlags(&R.shaded, cudaEventDisableTiming));
        KGK_CUDA(cudaEventCreateWithFlags(&R.shadowed, cudaEventDisableTiming));
    }
    // profile_stages == 2: stages one after another, so each stage time is its own
    const cudaStream_t sh_st = cfg->profile_stages == 2 ? st : R.st2;
    bool shadow_pending = false;  // shadow passes on st2 not yet waited for on st
    auto join_shadow = [&]() -> kgk_status {
        if (shadow_pending) KGK_CUDA(cudaStreamWaitEvent(st, R.shadowed, 0));
        shadow_pending = false;
        return KGK_OK;
    };
    cudaEvent_t e0, e1;
    KGK_CUDA(cudaEventCreate(&e0));
    KGK_CUDA(cudaEventCreate(&e1));
    KGK_CUDA(cudaEventRecord(e0, st));
    const int max_bounces = cfg->max_depth > 0 ? cfg->max_depth : 1024;
    uint64_t launches = 0, extend_launches = 0;
    // resident blocks per SM of the tail kernel used by this render
    int tail_blocks_per_sm = 1;
    {
        cudaError_t e;
        if (cfg->estimator == KGK_ESTIMATOR_COMPAT)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&tail_blocks_per_sm,
                                                              k_tail<KGK_ESTIMATOR_COMPAT, false>, 128, 0);
        else if (cfg->use_cache)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&tail_blocks_per_sm,
                                                              k_tail<KGK_ESTIMATOR_UNBIASED, true>, 128, 0);
        else
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&tail_blocks_per_sm,
                                                              k_tail<KGK_ESTIMATOR_UNBIASED, false>, 128, 0);
        KGK_CUDA(e);
        tail_blocks_per_sm = std::max(1, tail_blocks_per_sm);
    }
    // optional per-stage timing: an event before and after every stage launch
    const bool prof = cfg->profile_stages != 0;
    std::vector<cudaEvent_t> ev;
    std::vector<int> ev_stage;  // 0 extend, 1 shade, 2 shadow, 3 tail
    auto stage_begin = [&](int stage, cudaStream_t on = nullptr) -> kgk_status {
        if (!prof) return KGK_OK;
        cudaEvent_t a;
        KGK_CUDA(cudaEventCreate(&a));
        KGK_CUDA(cudaEventRecord(a, on ? on : st));
        ev.push_back(a);
        ev_stage.push_back(stage);
        return KGK_OK;
    };
    auto stage_end = [&](cudaStream_t on = nullptr) -> kgk_status {
        if (!prof) return KGK_OK;
        cudaEvent_t b;
        KGK_CUDA(cudaEventCreate(&b));
        KGK_CUDA(cudaEventRecord(b, on ? on : st));
        ev.push_back(b);
        ev_stage.push_back(-1);
        return KGK_OK;
    };
    for (int done = 0, wave = 0; done < cfg->spp; done += spw, ++wave) {
        P.spp_wave = std::min(spw, cfg->spp - done);
        P.sample_base = done;
        const int n = npx * P.spp_wave;
        if (P.use_cache) {
            KGK_CUDA(cudaMemsetAsync(R.cnt + kQN, 0, 2 * sizeof(int), st));
            if (wave > 0) P.train_stride = 0;  // training paths only in the first wave
        }
        P.cur = R.pb[0];
        P.nxt = R.pb[1];
        k_raygen<<<grid, 128, 0, st>>>(P);
        ++launches;
        auto launch_tail = [&](int cnt_idx, int dense_n, int bounces, int threads) -> kgk_status {
            KGK_TRY(stage_begin(3));
            const int tg = std::max(1, std::min((threads + 127) / 128, R.sms * tail_blocks_per_sm));
            KGK_CUDA(cudaMemsetAsync(R.cnt + kTF, 0, sizeof(int), st));
            if (cfg->estimator == KGK_ESTIMATOR_COMPAT) {
                k_tail<KGK_ESTIMATOR_COMPAT, false><<<tg, 128, 0, st>>>(P, cnt_idx, dense_n, bounces);
            } else {
                if (P.td_o) KGK_CUDA(cudaMemsetAsync(R.cnt + kTD, 0, 2 * sizeof(int), st));
                if (P.use_cache)
                    k_tail<KGK_ESTIMATOR_UNBIASED, true><<<tg, 128, 0, st>>>(P, cnt_idx, dense_n, bounces);
                else
                    k_tail<KGK_ESTIMATOR_UNBIASED, false><<<tg, 128, 0, st>>>(P, cnt_idx, dense_n, bounces);
                if (P.td_o) {
                    k_tail_shadow<<<grid, 128, 0, st>>>(P);
                    k_tail_resolve<<<tg, 128, 0, st>>>(P, cnt_idx, dense_n);
                    launches += 2;
                }
            }
            KGK_TRY(stage_end());
            KGK_CUDA(cudaGetLastError());
            ++launches;
            return KGK_OK;
        };
        // a small wave (the reference's estimator renders one sample per
        // pixel per wave) runs in the tail kernel from its primary rays
        bool drained = false;
        if (n <= kTailPaths) {
            KGK_TRY(launch_tail(-1, n, max_bounces, n));
            drained = true;
        }
        int c = 0;  // the buffer holding this bounce's live paths
        for (int b = 0; b < max_bounces && !drained; ++b) {
            P.cur = R.pb[c];
            P.nxt = R.pb[c ^ 1];
            const int cidx = b == 0 ? -1 : kA0 + c, nidx = kA0 + (c ^ 1);
            // extend's counters only: the previous bounce's shadow passes may still run
            KGK_CUDA(cudaMemsetAsync(R.cnt + kFE, 0, sizeof(int), st));
            KGK_CUDA(cudaMemsetAsync(R.cnt + kMQ, 0, (kDQ + 1 - kMQ) * sizeof(int), st));
            KGK_CUDA(cudaMemsetAsync(R.cnt + nidx, 0, sizeof(int), st));
            KGK_TRY(stage_begin(0));
            if (cfg->count_work)
                k_extend<true><<<grid, 128, 0, st>>>(P, cidx, n, R.mq, R.lq, R.dq);
            else
                k_extend<false><<<grid, 128, 0, st>>>(P, cidx, n, R.mq, R.lq, R.dq);
            KGK_TRY(stage_end());
            ++extend_launches;
            // shading adds to the radiance the previous shadow passes wrote and
            // refills their queues: wait for them, then reset the queue counters
            KGK_TRY(join_shadow());
            KGK_CUDA(cudaMemsetAsync(R.cnt + kSH0, 0, 2 * sizeof(int), st));
            KGK_CUDA(cudaMemsetAsync(R.cnt + kFS0, 0, 2 * sizeof(int), st));
            KGK_TRY(stage_begin(1));
            if (cfg->estimator == KGK_ESTIMATOR_COMPAT)
                k_shade<KGK_ESTIMATOR_COMPAT, false><<<grid, 128, 0, st>>>(P, R.mq, R.lq, R.dq, nidx, R.sh_o[0],
                                                                         R.sh_d[0], R.sh_c[0], R.sh_o[1], R.sh_d[1],
                                                                         R.sh_c[1]);
            else if (P.use_cache) {
                k_shade<KGK_ESTIMATOR_UNBIASED, true, 1><<<grid, 128, 0, st>>>(P, R.mq, R.lq, R.dq, nidx, R.sh_o[0],
                                                                             R.sh_d[0], R.sh_c[0], R.sh_o[1],
                                                                             R.sh_d[1], R.sh_c[1]);
                k_shade<KGK_ESTIMATOR_UNBIASED, true, 2><<<grid, 128, 0, st>>>(P, R.mq, R.lq, R.dq, nidx, R.sh_o[0],
                                                                             R.sh_d[0], R.sh_c[0], R.sh_o[1],
                                                                             R.sh_d[1], R.sh_c[1]);
                k_shade<KGK_ESTIMATOR_UNBIASED, true, 3><<<grid, 128, 0, st>>>(P, R.mq, R.lq, R.dq, nidx, R.sh_o[0],
                                                                             R.sh_d[0], R.sh_c[0], R.sh_o[1],
                                                                             R.sh_d[1], R.sh_c[1]);
                launches += 2;
            } else {  // without the cache, instances without its code
                k_shade<KGK_ESTIMATOR_UNBIASED, false, 1><<<grid, 128, 0, st>>>(P, R.mq, R.lq, R.dq, nidx, R.sh_o[0],
                                                                              R.sh_d[0], R.sh_c[0], R.sh_o[1],
                                                                              R.sh_d[1], R.sh_c[1]);
                k_shade<KGK_ESTIMATOR_UNBIASED, false, 2><<<grid, 128, 0, st>>>(P, R.mq, R.lq, R.dq, nidx, R.sh_o[0],
                                                                              R.sh_d[0], R.sh_c[0], R.sh_o[1],
                                                                              R.sh_d[1], R.sh_c[1]);
                k_shade<KGK_ESTIMATOR_UNBIASED, false, 3><<<grid, 128, 0, st>>>(P, R.mq, R.lq, R.dq, nidx, R.sh_o[0],
                                                                              R.sh_d[0], R.sh_c[0], R.sh_o[1],
                                                                              R.sh_d[1], R.sh_c[1]);
                launches += 2;
            }
            KGK_TRY(stage_end());
            KGK_CUDA(cudaEventRecord(R.shaded, st));
            KGK_CUDA(cudaStreamWaitEvent(sh_st, R.shaded, 0));
            KGK_TRY(stage_begin(2, sh_st));
            if (face_lights) {
                k_shadow<<<grid, 128, 0, sh_st>>>(P, kSH0, kFS0, R.sh_o[0], R.sh_d[0], R.sh_c[0]);
                ++launches;
            }
            k_shadow<<<grid, 128, 0, sh_st>>>(P, kSH1, kFS1, R.sh_o[1], R.sh_d[1], R.sh_c[1]);
            KGK_TRY(stage_end(sh_st));
            KGK_CUDA(cudaEventRecord(R.shadowed, sh_st));
            shadow_pending = true;
            KGK_CUDA(cudaGetLastError());
            launches += 3;
            c ^= 1;
            P.cur = R.pb[c];
            P.nxt = R.pb[c ^ 1];
            // from the second bounce on, check the live count every bounce,
            // to hand the last few paths to the tail kernel
            if (b >= 1) {
                int alive = 0;
                KGK_CUDA(cudaMemcpyAsync(&alive, R.cnt + kA0 + c, sizeof(int), cudaMemcpyDeviceToHost, st));
                KGK_CUDA(cudaStreamSynchronize(st));
                if (alive == 0) {
                    drained = true;
                    break;
                }
                if (alive <= kTailPaths && b + 1 < max_bounces) {
                    KGK_TRY(join_shadow());  // the tail starts from the radiance they complete
                    KGK_TRY(launch_tail(kA0 + c, 0, max_bounces - b - 1, alive));
                    drained = true;
                    break;
                }
            }
        }
        KGK_TRY(join_shadow());
        if (!drained) {
            // the bounce limit ended the wavefront with paths still live
            k_flush<<<grid, 128, 0, st>>>(P, kA0 + c);
            KGK_CUDA(cudaGetLastError());
            ++launches;
        }
        if (P.use_cache) {
            // terminate into the cache, then learn from this wave's training paths
            NrcState &N = *s->nrc;
            KGK_TRY(nrc_infer_dev(N, R.qrec, kQRec, R.cap, R.cnt + kQN, nullptr, R.fin, st));
            k_cache_targets<<<64, 256, 0, st>>>(R.trec, R.cnt + kTN, R.tcap, R.fin, R.ttgt);
            KGK_CUDA(cudaGetLastError());
            launches += 2;
            if (wave == 0) {
                int ntr = 0;
                KGK_CUDA(cudaMemcpyAsync(&ntr, R.cnt + kTN, sizeof(int), cudaMemcpyDeviceToHost, st));
                KGK_CUDA(cudaStreamSynchronize(st));
                ntr = std::min(ntr, R.tcap);
                if (ntr > 0) {
                    for (int k = 0; k < N.cfg.train_steps; ++k) {
                        KGK_TRY(nrc_grad_dev(N, R.trec, kQRec, R.ttgt, 3, ntr, nullptr, st));
                        KGK_TRY(nrc_step_dev(N, st));
                        launches += 6;
                    }
                }
            }
        }
        k_finish<<<(npx + 255) / 256, 256, 0, st>>>(P, R.frame, R.acc_sum, R.acc_sq, cfg->accumulate, wave == 0);
        KGK_CUDA(cudaGetLastError());
        ++launches;
    }
    if (cfg->accumulate) R.acc_n += (unsigned long long)cfg->spp;
    if (cfg->write_gbuffer) {
        R.gbuffer_valid = true;
        R.gbuffer_cam = *cam;
    }
    // output: the caller's device buffer, the scene's kept frame (out == NULL),
    // or staging copied to the caller's host buffer
    const bool od = out == nullptr || is_device_ptr(out);
    float4 *dout;
    R.kept_valid = out == nullptr;
    if (!out) {
        dout = R.kept;
    } else if (od) {
        dout = reinterpret_cast<float4 *>(out);
    } else {
        KGK_TRY(s->staging.reserve((size_t)npx * sizeof(float4)));
        dout = reinterpret_cast<float4 *>(s->staging.ptr);
    }
    k_output<<<(npx + 255) / 256, 256, 0, st>>>(R.frame, npx, 1.0f / (float)cfg->spp, dout);
    KGK_CUDA(cudaGetLastError());
    ++launches;
    KGK_CUDA(cudaEventRecord(e1, st));
    if (!od) KGK_CUDA(cudaMemcpyAsync(out, dout, (size_t)npx * sizeof(float4), cudaMemcpyDeviceToHost, st));
    unsigned long long hs[kNStat];
    KGK_CUDA(cudaMemcpyAsync(hs, R.stats, sizeof hs, cudaMemcpyDeviceToHost, st));
    KGK_CUDA(cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (stats) {
        memset(stats, 0, sizeof *stats);
        stats->rays_closest = hs[kRaysC];
        stats->rays_shadow = hs[kRaysS];
        stats->traversal_overflows = hs[kOverflow];
        stats->nodes_visited = hs[kNodes];
        stats->tris_tested = hs[kTris];
        stats->paths = (uint64_t)npx * (uint64_t)cfg->spp;
        stats->ms_device = ms;
        stats->kernel_launches = launches;
        stats->extend_launches = extend_launches;
        double stage_ms[4] = {0, 0, 0, 0};
        for (size_t k = 0; k + 1 < ev.size(); k += 2) {
            float m = 0;
            cudaEventElapsedTime(&m, ev[k], ev[k + 1]);
            stage_ms[ev_stage[k]] += m;
        }
        stats->ms_extend = stage_ms[0];
        stats->ms_shade = stage_ms[1];
        stats->ms_shadow = stage_ms[2];
        stats->ms_tail = stage_ms[3];
        stats->rays_tail = hs[kRaysT];
    }
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    if (cfg->use_cache) KGK_TRY(nrc_check_error(*s->nrc));
    if (hs[kOverflow])
        return fail(KGK_ERR_DEVICE_CHECK, "kgk_render: " + std::to_string(hs[kOverflow]) +
                                              " traversals overflowed their stack");
    return KGK_OK;
}

kgk_status kgk_accum_reset(kgk_scene *s, int32_t W, int32_t H) {
    if (!s) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_accum_reset: scene == NULL");
    if (W <= 0 || H <= 0 || (long long)W * H > (1LL << 26))
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_accum_reset: size out of range");
    KGK_CUDA(cudaSetDevice(s->device));
    RenderState &R = *render_state(s);
    const size_t n = (size_t)W * H * 3;
    if (R.acc_W != W || R.acc_H != H || !R.acc_sum) {
        KGK_TRY(ensure(&R.acc_sum, n, "FP64 accumulator"));
        KGK_TRY(ensure(&R.acc_sq, n, "FP64 accumulator"));
        R.acc_W = W;
        R.acc_H = H;
    }
    KGK_CUDA(cudaMemsetAsync(R.acc_sum, 0, n * sizeof(double), s->stream));
    KGK_CUDA(cudaMemsetAsync(R.acc_sq, 0, n * sizeof(double), s->stream));
    KGK_CUDA(cudaStreamSynchronize(s->stream));
    R.acc_n = 0;
    return KGK_OK;
}

kgk_status kgk_accum_read(kgk_scene *s, double *mean, double *var, uint64_t *n_samples) {
    if (!s || !mean) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_accum_read: NULL argument");
    RenderState *R = s->rs;
    if (!R || !R->acc_sum) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_accum_read: no accumulator (kgk_accum_reset)");
    KGK_CUDA(cudaSetDevice(s->device));
    const size_t n = (size_t)R->acc_W * R->acc_H * 3;
    std::vector<double> sum(n), sq(n);
    KGK_CUDA(cudaMemcpy(sum.data(), R->acc_sum, n * sizeof(double), cudaMemcpyDeviceToHost));
    KGK_CUDA(cudaMemcpy(sq.data(), R->acc_sq, n * sizeof(double), cudaMemcpyDeviceToHost));
    const double N = (double)R->acc_n;
    for (size_t i = 0; i < n; ++i) {
        const double m = N > 0 ? sum[i] / N : 0.0;
        mean[i] = m;
        if (var) var[i] = N > 1 ? std::max(0.0, (sq[i] - N * m * m) / (N - 1)) / N : 0.0;
    }
    if (n_samples) *n_samples = R->acc_n;
    return KGK_OK;
}

}  // extern "C"
