// svgf.cu - spatiotemporal variance-guided filtering.
//
// compat: ApplySVGF (SVGF.cuh:495-522) over the reference's own 112-byte
//   SVGFBuffer records.  Every __syncthreads of the reference, which it uses
//   as if it were a grid barrier, becomes a kernel boundary here, and reads
//   that precede a barrier while writes follow it are double-buffered: this
//   is the race-free reading of the filter, with its constants and quirks
//   (absolute pixel coordinates in the a-trous depth weight, SVGF.cuh:426;
//   the 5 x 5 stage loop, SVGF.cuh:486-491; the 0.2 blend, SVGF.cuh:459-464).
// standard: SVGF with reprojection of the previous frame from the previous
//   camera, temporal integration of colour and luminance moments (alpha),
//   spatial variance fallback, `atrous_iterations` edge-stopping a-trous
//   passes (sigma_z, sigma_n, sigma_l) on albedo-demodulated lighting, the
//   first pass feeding the next frame's history.
// temporal: the standard filter's reprojection and history alone, with
//   isolated outlier samples clamped before they enter the history and the
//   history clamped to the colour box of the current 3 x 3 neighbourhood.
#include <cmath>
#include <cstring>
#include <vector>

#include "kgk_device.cuh"
#include "kgk_scene.h"

static_assert(sizeof(kgk_svgf_buffer) == 112, "SVGFBuffer must be 112 B (struct_SVGFBuffers.cuh:7-23)");
static_assert(offsetof(kgk_svgf_buffer, ObjectID) == 64, "SVGFBuffer.ObjectID offset");
static_assert(offsetof(kgk_svgf_buffer, sampleNum) == 88, "SVGFBuffer.sampleNum offset");
static_assert(offsetof(kgk_svgf_buffer, Depth) == 104, "SVGFBuffer.Depth offset");
static_assert(offsetof(kgk_svgf_buffer, willApplyATrousFilter) == 108, "SVGFBuffer flag offset");

namespace kgk {

namespace {

constexpr float kS = 1e-4f;  // sINF

__device__ __forceinline__ float3 v3(kgk_vec v) { return f3(v.x, v.y, v.z); }
__device__ __forceinline__ kgk_vec kv(float3 a) { kgk_vec r; r.x = a.x; r.y = a.y; r.z = a.z; r.align = 0.0f; return r; }
__device__ __forceinline__ float lumf(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
__device__ __forceinline__ float3 div3(float3 a, float3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }

__device__ __forceinline__ void sb_init(kgk_svgf_buffer &b) {
    const kgk_vec z = {0, 0, 0, 0};
    b.Albedo = b.Emission = b.Normal = b.ColorHistory = z;
    b.ObjectID = -1;
    b.MaterialID = -1;
    b.PosLastFrameI[0] = b.PosLastFrameI[1] = -1;
    b.PosLastFrameF[0] = b.PosLastFrameF[1] = -1.0f;
    b.sampleNum = 0;
    b.MomentOne = -1.0f;
    b.MomentTwo = -1.0f;
    b.Variance = 0.0f;
    b.Depth = 0.0f;
    b.willApplyATrousFilter = true;
    b.willApplyTemporalAccumulation = false;
}

__device__ __forceinline__ float depth_w(float d, float nd, int dx, int dy, float gx, float gy) {
    const float top = -1.0f * fabsf(d - nd);
    const float bottom = 1.0f * fabsf((float)dx * gx + (float)dy * gy) + kS;
    return expf(top / bottom);
}
__device__ __forceinline__ float normal_w(float3 n, float3 m) {
    float c = fmaxf(0.0f, dot3(n, m));
    c *= c; c *= c; c *= c; c *= c; c *= c; c *= c; c *= c;  // ^128
    return c;
}
__device__ __forceinline__ float lum_w(float l, float nl, float sd) {
    const float top = -1.0f * fabsf(l - nl);
    const float bottom = 4.0f * sd + kS;
    return expf(top / bottom);
}

struct CompatArgs {
    int W, H, frame;
    kgk_vec *R, *F;
    kgk_svgf_buffer *P, *C;
    float *M1, *M2, *sd, *gz, *s1, *s2, *sw, *var;
    unsigned char *spatial;
    kgk_vec *R2;
    // the a-trous passes' per-pixel guide, packed from the records once their
    // fields are final (k_c_gauss2): normal and depth, ObjectID and MaterialID
    float4 *gnd;
    int2 *gom;
    // the center pixel's albedo and willApplyATrousFilter (w = 1 or 0),
    // final from k_c_gauss2 on: a pass reads 16 B instead of two sectors of
    // the 112-byte record
    float4 *galf;
    // each pass's input radiance divided by (albedo + sINF), with its
    // luminance in w: written by the pass before (ping-pong), so a tap reads
    // it instead of dividing
    float4 *dm, *dm2;
};

#define FOR_PIXELS(n) for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < (n); p += gridDim.x * blockDim.x)

// save_png's tone mapping on the device.  tone_host's bytes are a step
// function of x; T holds its 255 steps (the smallest x reaching each byte,
// computed with the host's powf), so counting the steps at or below x gives
// tone_host(x) exactly.  NaN and negative x give 0 (powf is NaN there), except
// -inf, where powf(-inf, 1/2.2f) = +inf gives 255.
struct ToneTable {
    float t[255];
};

__device__ __forceinline__ unsigned tone_byte(float x, const ToneTable &T) {
    if (!(x >= 0.0f)) return x == -__int_as_float(0x7f800000) ? 255u : 0u;
    unsigned i = 0;
#pragma unroll
    for (unsigned step = 128; step; step >>= 1)
        if (T.t[i + step - 1] <= x) i += step;
    return i;
}

__device__ __forceinline__ uchar4 tone_rgba8(float4 c, const ToneTable &T) {
    return make_uchar4((unsigned char)tone_byte(c.x, T), (unsigned char)tone_byte(c.y, T),
                       (unsigned char)tone_byte(c.z, T), 255);
}

__global__ void k_tonemap(const float4 *__restrict__ in, size_t npx, uchar4 *__restrict__ out,
                          const __grid_constant__ ToneTable T) {
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < npx; p += (size_t)gridDim.x * blockDim.x)
        out[p] = tone_rgba8(in[p], T);
}

ToneTable tone_table() {
    ToneTable T;
    memcpy(T.t, tone_thresholds(), sizeof T.t);
    return T;
}

__global__ void k_c_prologue(CompatArgs a) {
    FOR_PIXELS(a.W * a.H) {
        float3 r = v3(a.R[p]);
        if (!isfinite(len3(r))) a.R[p] = kv(f3(0.0f, 0.0f, 0.0f));
        if (a.frame == 0) sb_init(a.P[p]);
        if (a.P[p].MomentOne == -1.0f) {
            const float m1 = lumf(div3(v3(a.R[p]), v3(a.C[p].Albedo)));
            a.C[p].MomentOne = m1;
            a.C[p].MomentTwo = m1 * m1;
        }
        a.F[p] = kv(f3(0.0f, 0.0f, 0.0f));
    }
}

// TemporalAccumulation (SVGF.cuh:50-98)
__global__ void k_c_temporal(CompatArgs a) {
    const int W = a.W, H = a.H;
    FOR_PIXELS(W * H) {
        const kgk_svgf_buffer &c = a.C[p];
        if (len3(v3(c.Emission)) != 0.0f) continue;
        const int px = c.PosLastFrameI[0], py = c.PosLastFrameI[1];
        const float s = c.PosLastFrameF[0] - (float)px, t = c.PosLastFrameF[1] - (float)py;
        const int ox[4] = {0, 1, 0, 1}, oy[4] = {0, 0, 1, 1};
        const float w[4] = {(1 - s) * (1 - t), s * (1 - t), (1 - s) * t, s * t};
        float3 sum = f3(0.0f, 0.0f, 0.0f);
        float swt = 0.0f;
        for (int i = 0; i < 4; ++i) {
            const int qx = px + ox[i], qy = py + oy[i];
            if (qx < 0 || qx >= W || qy < 0 || qy >= H) continue;
            const kgk_svgf_buffer &q = a.P[W * qy + qx];
            if (q.MaterialID == c.MaterialID && q.willApplyTemporalAccumulation) {
                sum += v3(q.ColorHistory) * w[i];
                swt += w[i];
            }
        }
        if (swt == 0.0f) continue;
        const float3 hist = sum / swt;
        a.R[p] = kv(v3(a.R[p]) * 0.2f + hist * 0.8f);
    }
}

// VarianceEstimation, before the first barrier (SVGF.cuh:114-145)
__global__ void k_c_var1(CompatArgs a) {
    const int W = a.W, H = a.H;
    FOR_PIXELS(W * H) {
        const int x = p % W, y = p / W;
        const kgk_svgf_buffer &c = a.C[p];
        const float l = lumf(div3(v3(a.R[p]), v3(c.Albedo) + f3(kS, kS, kS)));
        a.M1[p] = l;
        a.M2[p] = l * l;
        bool sp = c.PosLastFrameI[0] == -1;
        if (!sp) {
            const int prev = W * c.PosLastFrameI[1] + c.PosLastFrameI[0];
            sp = (prev < 0 || prev >= W * H) ? true : a.P[prev].sampleNum < 3;
        }
        a.spatial[p] = sp ? 1 : 0;
        const int dx = x < W / 2 ? 1 : -1, dy = y < H / 2 ? 1 : -1;
        const float d = c.Depth;
        a.gz[2 * p] = (a.C[W * y + x + dx].Depth - d) / (float)dx;
        a.gz[2 * p + 1] = (a.C[W * (y + dy) + x].Depth - d) / (float)dy;
        // the guide k_c_var3 reads (the records as they are before k_c_var4)
        a.gnd[p] = make_float4(c.Normal.x, c.Normal.y, c.Normal.z, d);
        a.gom[p] = make_int2(c.ObjectID, c.MaterialID);
    }
}

__global__ void k_c_var2(CompatArgs a) {
    const int W = a.W;
    FOR_PIXELS(W * a.H) {
        if (a.spatial[p]) continue;
        kgk_svgf_buffer &c = a.C[p];
        const int prev = W * c.PosLastFrameI[1] + c.PosLastFrameI[0];
        c.sampleNum = a.P[prev].sampleNum + 1;
        float cw = 1.0f / 5.0f;
        if (c.sampleNum < 5) cw = 1.0f / (float)c.sampleNum;
        c.MomentOne = (1.0f - cw) * a.P[prev].MomentOne + cw * a.M1[p];
        c.MomentTwo = (1.0f - cw) * a.P[prev].MomentTwo + cw * a.M2[p];
        a.M1[p] = c.MomentOne;
        a.M2[p] = c.MomentTwo;
    }
}

__constant__ float cK7[7] = {0.00598f, 0.060626f, 0.241843f, 0.383103f, 0.241843f, 0.060626f, 0.00598f};
__constant__ float cKG[3] = {1 / 4.0f, 1 / 2.0f, 1 / 4.0f};
__constant__ float cKW[25] = {1 / 256.0f, 4 / 256.0f, 6 / 256.0f, 4 / 256.0f, 1 / 256.0f,
                              4 / 256.0f, 16 / 256.0f, 24 / 256.0f, 16 / 256.0f, 4 / 256.0f,
                              6 / 256.0f, 24 / 256.0f, 36 / 256.0f, 24 / 256.0f, 6 / 256.0f,
                              4 / 256.0f, 16 / 256.0f, 24 / 256.0f, 16 / 256.0f, 4 / 256.0f,
                              1 / 256.0f, 4 / 256.0f, 6 / 256.0f, 4 / 256.0f, 1 / 256.0f};

// 7x7 edge-stopped moment filter (SVGF.cuh:166-225) on 32 x 8-pixel tiles:
// a block stages the guide, ids and moments of its pixels and a halo of 3,
// then sums in the reference's order (kx outer, ky inner).
constexpr int kCTX = 32, kCTY = 8;
__global__ void __launch_bounds__(256) k_c_var3(CompatArgs a) {
    constexpr int R = 3, SX = kCTX + 2 * R, SY = kCTY + 2 * R;
    __shared__ float4 s_nd[SY * SX];
    __shared__ int2 s_om[SY * SX];
    __shared__ float2 s_m[SY * SX];
    const int W = a.W, H = a.H;
    const int x0 = blockIdx.x * kCTX - R, y0 = blockIdx.y * kCTY - R;
    for (int i = threadIdx.y * kCTX + threadIdx.x; i < SX * SY; i += kCTX * kCTY) {
        const int gx = x0 + i % SX, gy = y0 + i / SX;
        if (gx < 0 || gx >= W || gy < 0 || gy >= H) continue;
        const int q = W * gy + gx;
        s_nd[i] = a.gnd[q];
        s_om[i] = a.gom[q];
        s_m[i] = make_float2(a.M1[q], a.M2[q]);
    }
    __syncthreads();
    const int x = blockIdx.x * kCTX + threadIdx.x, y = blockIdx.y * kCTY + threadIdx.y;
    if (x >= W || y >= H) return;
    const int p = W * y + x, c = SX * (threadIdx.y + R) + threadIdx.x + R;
    a.sw[p] = a.s1[p] = a.s2[p] = 0.0f;
    if (!a.spatial[p]) return;
    const float4 cn = s_nd[c];
    const int cmat = s_om[c].y;
    const float3 n = f3(cn);
    const float gzx = a.gz[2 * p], gzy = a.gz[2 * p + 1];
    float s1 = 0, s2 = 0, sw = 0;
    for (int kx = -3; kx <= 3; ++kx) {
        const int nx = x + kx;
        if (nx < 0 || nx >= W) continue;
        const float hx = cK7[kx + 3];
        for (int ky = -3; ky <= 3; ++ky) {
            const int ny = y + ky;
            if (ny < 0 || ny >= H) continue;
            const float hy = cK7[ky + 3];
            if (kx == 0 && ky == 0) {
                s1 += hx * hy * s_m[c].x;
                s2 += hx * hy * s_m[c].y;
                sw += hx * hy;
                continue;
            }
            const int t = c + SX * ky + kx;
            const int2 om = s_om[t];
            if (om.x == -1) continue;
            const float4 qn = s_nd[t];
            const float wm = cmat == om.y ? 1.0f : 0.0f;
            const float wz = depth_w(cn.w, qn.w, kx, ky, gzx, gzy);
            const float wn = normal_w(n, f3(qn));
            const float w = hx * hy * wz * wn * wm;
            s1 += w * s_m[t].x;
            s2 += w * s_m[t].y;
            sw += w;
        }
    }
    a.s1[p] = s1;
    a.s2[p] = s2;
    a.sw[p] = sw;
}

__global__ void k_c_var4(CompatArgs a) {
    const int W = a.W;
    FOR_PIXELS(W * a.H) {
        kgk_svgf_buffer &c = a.C[p];
        if (c.ObjectID == -1 || (a.spatial[p] && a.sw[p] == 0.0f)) {
            a.F[p] = a.R[p];
            sb_init(c);
            c.willApplyATrousFilter = false;
        } else if (a.spatial[p]) {
            c.MomentOne = a.s1[p] / a.sw[p];
            c.MomentTwo = a.s2[p] / a.sw[p];
            if (c.PosLastFrameI[0] == -1) c.sampleNum = 1;
            else c.sampleNum = a.P[W * c.PosLastFrameI[1] + c.PosLastFrameI[0]].sampleNum + 1;
        }
    }
}

__global__ void k_c_var5(CompatArgs a) {
    FOR_PIXELS(a.W * a.H) {
        kgk_svgf_buffer &c = a.C[p];
        if (c.ObjectID == -1) continue;
        c.Variance = fmaxf(0.0f, c.MomentTwo - c.MomentOne * c.MomentOne);
        if (c.Variance > 1000) c.Variance = 1000;
    }
}

// ApplyGaussianFilterToVar (SVGF.cuh:277-344)
__global__ void k_c_gauss1(CompatArgs a) {
    const int W = a.W, H = a.H;
    FOR_PIXELS(W * H) {
        const int x = p % W, y = p / W;
        float sv = 0, sw = 0;
        for (int kx = -1; kx <= 1; ++kx) {
            const float hx = cKG[kx + 1];
            const int nx = x + kx;
            if (nx < 0 || nx >= W) continue;
            for (int ky = -1; ky <= 1; ++ky) {
                const float hy = cKG[ky + 1];
                const int ny = y + ky;
                if (ny < 0 || ny >= H) continue;
                const kgk_svgf_buffer &d = a.C[W * ny + nx];
                if (d.ObjectID == -1) continue;
                const float w = hx * hy;
                sv += w * d.Variance;
                sw += w;
            }
        }
        a.s1[p] = sv;
        a.sw[p] = sw;
    }
}

__global__ void k_c_gauss2(CompatArgs a) {
    FOR_PIXELS(a.W * a.H) {
        kgk_svgf_buffer &c = a.C[p];
        a.sd[p] = 0.0f;
        if (a.s1[p] == 0.0f && a.sw[p] != 0.0f) {
            a.F[p] = a.R[p];
            c.willApplyATrousFilter = false;
        } else if (a.sw[p] == 0.0f) {
            c.MomentOne = -1.0f;
            c.MomentTwo = -1.0f;
            c.sampleNum = 0;
            c.willApplyATrousFilter = false;
        } else {
            c.Variance = a.s1[p] / a.sw[p];
            a.sd[p] = sqrtf(a.s1[p] / a.sw[p]);
        }
        a.var[p] = c.Variance;
        // the records' normal, depth, ids and albedo are final from here to
        // the end of the a-trous passes, and so is R before the first pass
        a.gnd[p] = make_float4(c.Normal.x, c.Normal.y, c.Normal.z, c.Depth);
        a.gom[p] = make_int2(c.ObjectID, c.MaterialID);
        a.galf[p] = make_float4(c.Albedo.x, c.Albedo.y, c.Albedo.z, c.willApplyATrousFilter ? 1.0f : 0.0f);
        const float3 dc = div3(v3(a.R[p]), v3(c.Albedo) + f3(kS, kS, kS));
        a.dm[p] = make_float4(dc.x, dc.y, dc.z, lumf(dc));
        // the a-trous passes' depth gradient (SVGF.cuh:366-372), from the
        // records as k_c_var4 left them; k_c_var3 was the last reader of gz
        const int W = a.W, x = p % W, y = p / W;
        const int dx = x < W / 2 ? 1 : -1, dy = y < a.H / 2 ? 1 : -1;
        a.gz[2 * p] = (a.C[W * y + x + dx].Depth - c.Depth) / (float)dx;
        a.gz[2 * p + 1] = (a.C[W * (y + dy) + x].Depth - c.Depth) / (float)dy;
    }
}

// One a-trous stage (SVGF.cuh:347-474) of pixel p = (x, y) at step 2^stage.
// Reads go through Src: the global arrays (k_c_atrous) or a shared-memory
// tile of them (k_c_atrous_tile); either way every tap is the reference's
// expression in its order, so both give the same bits.  A tap's neighbour
// radiance comes demodulated with its luminance (dm, written by the pass
// before) instead of being divided by its albedo at every tap.
struct CompatIO {
    const kgk_vec *Rin;
    kgk_vec *Rout;
    const float4 *dmin;
    float4 *dmout;
    const float *vin;
    float *vout;
};

template <class Src>
__device__ __forceinline__ void compat_atrous_px(const CompatArgs &a, const CompatIO &io, const Src &S, int x, int y,
                                                 int stage) {
    const int W = a.W, H = a.H, p = W * y + x, step = 1 << stage;
    const float4 af = a.galf[p];
    const float4 g = S.nd(0, 0);
    const int2 om = S.om(0, 0);
    const float4 dcl = S.dm(0, 0);
    const float3 dc = f3(dcl);
    const float l = dcl.w;
    const float d = g.w;
    const float gx = a.gz[2 * p], gy = a.gz[2 * p + 1];
    const float3 n = f3(g);
    const float sdv = a.sd[p];
    const bool filt = af.w != 0.0f;
    float3 srad = f3(0.0f, 0.0f, 0.0f);
    float svar = 0.0f, swt = 0.0f;
#pragma unroll
    for (int ki = 0; ki < 25; ++ki) {
        const float h = cKW[ki];
        const int ox = (ki % 5 - 2) * step, oy = (ki / 5 - 2) * step;
        const int qx = x + ox, qy = y + oy;
        if (qx < 0 || qx >= W || qy < 0 || qy >= H) continue;
        if (ki == 12) {
            svar += h * h * S.v(0, 0);
            srad += dc * h;
            swt += h;
            continue;
        }
        const int2 eo = S.om(ox, oy);
        if (eo.x == -1) continue;
        const float4 em = S.dm(ox, oy);
        const float3 nr = f3(em);
        const float nl = em.w;
        if (((double)l > 0.5 && nl > 5 * l) || ((double)l > 0.1 && nl > 50 * l) || (l > kS && nl > 100 * l))
            continue;
        const float4 eg = S.nd(ox, oy);
        const float wm = om.y == eo.y ? 1.0f : 0.0f;
        const float wz = depth_w(d, eg.w, qx, qy, gx, gy);  // absolute coordinates, SVGF.cuh:426
        const float wn = normal_w(n, f3(eg));
        const float wl = lum_w(l, nl, sdv);
        const float w = filt ? h * wz * wn * wl * wm : h * wz * wn * wm;
        srad += nr * w;
        svar += w * w * S.v(ox, oy);
        swt += w;
    }
    const kgk_vec rin = io.Rin[p];
    const float vc = S.v(0, 0);
    if (om.x == -1 || swt < 1e-6f || swt * swt < 1e-6f) {
        io.Rout[p] = rin;
        io.vout[p] = vc;
        io.dmout[p] = dcl;
        if (om.x == -1) return;
        a.F[p] = rin;
        a.C[p].willApplyTemporalAccumulation = true;
        return;
    }
    const float3 alb = f3(af);
    const float3 fl = srad / swt;
    const float fv = svar / (swt * swt);
    const float cw = 0.2f;
    const float3 o = (fl * alb) * cw + v3(rin) * (1 - cw);
    a.F[p] = kv(o);
    io.Rout[p] = kv(o);
    const float3 od = div3(o, alb + f3(kS, kS, kS));
    io.dmout[p] = make_float4(od.x, od.y, od.z, lumf(od));
    io.vout[p] = filt ? cw * vc + (1 - cw) * fv : vc;
    if (stage == 0) {
        a.C[p].ColorHistory = kv(o);
        a.C[p].willApplyTemporalAccumulation = true;
    }
}

// Taps read straight from the global arrays (offsets from pixel p).
struct CompatGlobal {
    const float4 *gnd_, *dm_;
    const int2 *gom_;
    const float *v_;
    int p, W;
    __device__ float4 nd(int ox, int oy) const { return gnd_[p + W * oy + ox]; }
    __device__ int2 om(int ox, int oy) const { return gom_[p + W * oy + ox]; }
    __device__ float4 dm(int ox, int oy) const { return dm_[p + W * oy + ox]; }
    __device__ float v(int ox, int oy) const { return v_[p + W * oy + ox]; }
};

__global__ void k_c_atrous(CompatArgs a, CompatIO io, int stage) {
    const int W = a.W;
    FOR_PIXELS(W * a.H) {
        const CompatGlobal S{a.gnd, io.dmin, a.gom, io.vin, p, W};
        compat_atrous_px(a, io, S, p % W, p / W, stage);
    }
}

// The same stage for steps 1, 2 and 4 on 32 x 8-pixel tiles: a block stages
// its pixels and a halo of 2 * step (all 25 taps and the depth gradient's
// neighbours) in shared memory - guide, ids, demodulated radiance, variance -
// then filters from there.  Entries outside the image are never read (the
// tap's bounds test comes first).
template <int kStep> struct CTile {
    static constexpr int R = 2 * kStep, SX = kCTX + 2 * R, SY = kCTY + 2 * R, N = SX * SY;
    static constexpr size_t kSmem = (size_t)N * (2 * sizeof(float4) + sizeof(int2) + sizeof(float));
};

// Taps read from a tile of row length SX (offsets from entry c).
template <int SX> struct CompatShared {
    const float4 *snd, *sdm;
    const int2 *som;
    const float *sv;
    int c;
    __device__ float4 nd(int ox, int oy) const { return snd[c + SX * oy + ox]; }
    __device__ int2 om(int ox, int oy) const { return som[c + SX * oy + ox]; }
    __device__ float4 dm(int ox, int oy) const { return sdm[c + SX * oy + ox]; }
    __device__ float v(int ox, int oy) const { return sv[c + SX * oy + ox]; }
};

template <int kStep>
__global__ void __launch_bounds__(256) k_c_atrous_tile(CompatArgs a, CompatIO io) {
    using T = CTile<kStep>;
    extern __shared__ __align__(16) unsigned char smem[];
    float4 *s_nd = (float4 *)smem;
    float4 *s_dm = s_nd + T::N;
    int2 *s_om = (int2 *)(s_dm + T::N);
    float *s_v = (float *)(s_om + T::N);
    const int W = a.W, H = a.H;
    const int x0 = blockIdx.x * kCTX - T::R, y0 = blockIdx.y * kCTY - T::R;
    for (int i = threadIdx.y * kCTX + threadIdx.x; i < T::N; i += kCTX * kCTY) {
        const int gx = x0 + i % T::SX, gy = y0 + i / T::SX;
        if (gx < 0 || gx >= W || gy < 0 || gy >= H) continue;
        const int q = W * gy + gx;
        s_nd[i] = a.gnd[q];
        s_dm[i] = io.dmin[q];
        s_om[i] = a.gom[q];
        s_v[i] = io.vin[q];
    }
    __syncthreads();
    const int x = blockIdx.x * kCTX + threadIdx.x, y = blockIdx.y * kCTY + threadIdx.y;
    if (x >= W || y >= H) return;
    const CompatShared<T::SX> S{s_nd, s_dm, s_om, s_v, T::SX * ((int)threadIdx.y + T::R) + (int)threadIdx.x + T::R};
    compat_atrous_px(a, io, S, x, y, kStep == 1 ? 0 : kStep == 2 ? 1 : 2);
}

// The same stage for steps of 8 and more on row segments: a block of 256
// threads takes 256 pixels of one row and stages the five rows its taps read
// (y + {-2, -1, 0, 1, 2} step), each 256 + 4 step entries wide, so that every
// tap comes from shared memory and the staging reads are coalesced.
template <int kStep> struct CRows {
    static constexpr int T = 256, R = 2 * kStep, SX = T + 2 * R, N = 5 * SX;
    static constexpr size_t kSmem = (size_t)N * (2 * sizeof(float4) + sizeof(int2) + sizeof(float));
};

// Taps read from the five staged rows (row pitch SX, one row per step).
template <int SX, int kStep> struct CompatRows {
    const float4 *snd, *sdm;
    const int2 *som;
    const float *sv;
    int c;
    __device__ int at(int ox, int oy) const { return c + SX * (oy / kStep) + ox; }
    __device__ float4 nd(int ox, int oy) const { return snd[at(ox, oy)]; }
    __device__ int2 om(int ox, int oy) const { return som[at(ox, oy)]; }
    __device__ float4 dm(int ox, int oy) const { return sdm[at(ox, oy)]; }
    __device__ float v(int ox, int oy) const { return sv[at(ox, oy)]; }
};

template <int kStep>
__global__ void __launch_bounds__(256) k_c_atrous_rows(CompatArgs a, CompatIO io) {
    using T = CRows<kStep>;
    extern __shared__ __align__(16) unsigned char smem[];
    float4 *s_nd = (float4 *)smem;
    float4 *s_dm = s_nd + T::N;
    int2 *s_om = (int2 *)(s_dm + T::N);
    float *s_v = (float *)(s_om + T::N);
    const int W = a.W, H = a.H, y = blockIdx.y;
    const int x0 = blockIdx.x * T::T - T::R;
    for (int i = threadIdx.x; i < T::N; i += T::T) {
        const int gx = x0 + i % T::SX, gy = y + (i / T::SX - 2) * kStep;
        if (gx < 0 || gx >= W || gy < 0 || gy >= H) continue;
        const int q = W * gy + gx;
        s_nd[i] = a.gnd[q];
        s_dm[i] = io.dmin[q];
        s_om[i] = a.gom[q];
        s_v[i] = io.vin[q];
    }
    __syncthreads();
    const int x = blockIdx.x * T::T + threadIdx.x;
    if (x >= W) return;
    constexpr int stage = kStep == 8 ? 3 : kStep == 16 ? 4 : kStep == 32 ? 5 : 6;
    static_assert((1 << stage) == kStep, "row-tile steps are 8, 16, 32 and 64");
    const CompatRows<T::SX, kStep> S{s_nd, s_dm, s_om, s_v, 2 * T::SX + (int)threadIdx.x + T::R};
    compat_atrous_px(a, io, S, x, y, stage);
}

__global__ void k_c_final(CompatArgs a, const float *var) {
    FOR_PIXELS(a.W * a.H) {
        a.C[p].Variance = var[p];
        a.R[p] = a.C[p].ColorHistory;
    }
}

__global__ void k_copy_vec(const kgk_vec *src, kgk_vec *dst, int n) {
    FOR_PIXELS(n) dst[p] = src[p];
}

// Scratch of the compat pipeline, carved from one block: M1, M2, sd, gz (two
// arrays), s1, s2, sw, var, var2 at `fl` bytes each, then R2 (`vec` bytes),
// the guide (gnd, 16 B a pixel), the two demodulated radiance buffers (dm,
// dm2, 16 B each), albedo + filter flag (galf, 16 B), the ids (gom, 8 B),
// then the per-pixel spatial flags;
// every array starts on a 256-byte boundary.  Returns var2, the second
// variance buffer of the a-trous passes.
constexpr size_t scratch_up(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t compat_fl(size_t npx) { return scratch_up(npx * sizeof(float)); }
constexpr size_t compat_vec(size_t npx) { return scratch_up(npx * sizeof(kgk_vec)); }
constexpr size_t compat_scratch_bytes(size_t npx) {
    return 10 * compat_fl(npx) + 5 * compat_vec(npx) + scratch_up(npx * sizeof(int2)) + npx;
}

float *carve_compat(CompatArgs &a, unsigned char *b, size_t fl, size_t vec) {
    a.M1 = (float *)b; b += fl;
    a.M2 = (float *)b; b += fl;
    a.sd = (float *)b; b += fl;
    a.gz = (float *)b; b += 2 * fl;
    a.s1 = (float *)b; b += fl;
    a.s2 = (float *)b; b += fl;
    a.sw = (float *)b; b += fl;
    a.var = (float *)b; b += fl;
    float *var2 = (float *)b; b += fl;
    a.R2 = (kgk_vec *)b; b += vec;
    a.gnd = (float4 *)b; b += vec;
    a.dm = (float4 *)b; b += vec;
    a.dm2 = (float4 *)b; b += vec;
    a.galf = (float4 *)b; b += vec;
    a.gom = (int2 *)b; b += scratch_up(vec / 2);
    a.spatial = b;
    return var2;
}

// Queues the compat pipeline (SVGF.cuh:495-522, every __syncthreads a kernel
// boundary) on `st` and waits for it.  Every scratch word is written by an
// earlier kernel of the same call before any kernel reads it.
kgk_status launch_compat(CompatArgs &a, float *var2, int repeats, int stages, cudaStream_t st) {
    const size_t npx = (size_t)a.W * a.H;
    const int g = (int)std::min<size_t>((npx + 255) / 256, 65535);
    KGK_CUDA(cudaFuncSetAttribute(k_c_atrous_tile<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)CTile<4>::kSmem));
    KGK_CUDA(cudaFuncSetAttribute(k_c_atrous_rows<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)CRows<8>::kSmem));
    KGK_CUDA(cudaFuncSetAttribute(k_c_atrous_rows<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)CRows<16>::kSmem));
    k_c_prologue<<<g, 256, 0, st>>>(a);
    k_c_temporal<<<g, 256, 0, st>>>(a);
    k_c_var1<<<g, 256, 0, st>>>(a);
    k_c_var2<<<g, 256, 0, st>>>(a);
    const dim3 tiles((a.W + kCTX - 1) / kCTX, (a.H + kCTY - 1) / kCTY), tile_threads(kCTX, kCTY);
    k_c_var3<<<tiles, tile_threads, 0, st>>>(a);
    k_c_var4<<<g, 256, 0, st>>>(a);
    k_c_var5<<<g, 256, 0, st>>>(a);
    k_c_gauss1<<<g, 256, 0, st>>>(a);
    k_c_gauss2<<<g, 256, 0, st>>>(a);
    kgk_vec *rin = a.R, *rout = a.R2;
    float4 *din = a.dm, *dout = a.dm2;
    float *vin = a.var, *vout = var2;
    for (int k = 0; k < repeats; ++k)
        for (int s = 0; s < stages; ++s) {
            const CompatIO io{rin, rout, din, dout, vin, vout};
            const dim3 rows((a.W + 255) / 256, a.H);
            switch (s) {
                case 0: k_c_atrous_tile<1><<<tiles, tile_threads, CTile<1>::kSmem, st>>>(a, io); break;
                case 1: k_c_atrous_tile<2><<<tiles, tile_threads, CTile<2>::kSmem, st>>>(a, io); break;
                case 2: k_c_atrous_tile<4><<<tiles, tile_threads, CTile<4>::kSmem, st>>>(a, io); break;
                case 3: k_c_atrous_rows<8><<<rows, 256, CRows<8>::kSmem, st>>>(a, io); break;
                case 4: k_c_atrous_rows<16><<<rows, 256, CRows<16>::kSmem, st>>>(a, io); break;
                default: k_c_atrous<<<g, 256, 0, st>>>(a, io, s); break;
            }
            std::swap(rin, rout);
            std::swap(din, dout);
            std::swap(vin, vout);
        }
    if (rin != a.R) k_copy_vec<<<g, 256, 0, st>>>(rin, a.R, (int)npx);
    k_c_final<<<g, 256, 0, st>>>(a, vin);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "SVGF compat kernels");
    return KGK_OK;
}

// Runs the compat pipeline on device buffers (R, F, P, C all W*H records),
// with `scratch` (compat_scratch_bytes(W * H)), or scratch allocated for the
// call when it is null.
kgk_status run_compat(kgk_vec *R, kgk_vec *F, kgk_svgf_buffer *P, kgk_svgf_buffer *C, int W, int H, int frame,
                      int repeats, int stages, cudaStream_t st, unsigned char *scratch = nullptr) {
    const size_t npx = (size_t)W * H;
    void *owned = nullptr;
    if (!scratch) {
        KGK_TRY(dmalloc(&owned, compat_scratch_bytes(npx), "SVGF scratch"));
        scratch = (unsigned char *)owned;
    }
    CompatArgs a;
    a.W = W; a.H = H; a.frame = frame; a.R = R; a.F = F; a.P = P; a.C = C;
    float *var2 = carve_compat(a, scratch, compat_fl(npx), compat_vec(npx));
    const kgk_status stt = launch_compat(a, var2, repeats, stages, st);
    if (owned) dfree(owned);
    return stt;
}

// Fills reference-layout records from the renderer's G-buffer, the way
// render.cuh:28 (init) and RayTrace.cuh:66-82 fill them.  A block builds its
// 256 records in shared memory and writes them out as consecutive words, so
// that the 112-byte records are stored with coalesced writes.
constexpr int kRecWords = (int)(sizeof(kgk_svgf_buffer) / 4);
__global__ void __launch_bounds__(256) k_gbuffer_to_records(const float4 *pos, const float4 *nrm, const float4 *alb,
                                                            const float4 *emi, size_t npx, kgk_svgf_buffer *C) {
    __shared__ __align__(16) unsigned s_rec[256 * kRecWords];
    const size_t base = (size_t)blockIdx.x * 256;
    const int n = (int)min((size_t)256, npx - base);
    if ((int)threadIdx.x < n) {
        const size_t p = base + threadIdx.x;
        kgk_svgf_buffer b;
        sb_init(b);
        const float4 nr = nrm[p];
        const int obj = __float_as_int(nr.w);
        if (obj >= 0) {
            const float4 al = alb[p];
            b.Albedo = kv(f3(al));
            b.Emission = kv(f3(emi[p]));
            b.Normal = kv(f3(nr));
            b.ObjectID = obj;
            b.MaterialID = __float_as_int(al.w);
            b.Depth = pos[p].w;
        }
        *reinterpret_cast<kgk_svgf_buffer *>(s_rec + threadIdx.x * kRecWords) = b;
    }
    __syncthreads();
    unsigned *dst = reinterpret_cast<unsigned *>(C + base);
    for (int i = threadIdx.x; i < n * kRecWords; i += 256) dst[i] = s_rec[i];
}

// ---------------------------------------------------------------------------
// standard SVGF
// ---------------------------------------------------------------------------
struct StdArgs {
    int W, H;
    const float4 *pos, *nrm, *alb, *emi;   // current G-buffer
    const float4 *noisy;                   // current frame (kgk_vec)
    float4 *hist, *hist_prev;
    float2 *mom, *mom_prev;
    float4 *nd, *nd_prev;                  // normal + depth, this frame (written by k_s_temporal) and the last
    int *mat, *mat_prev;                   // material id (>= 0) or -1 for no hit, same
    float *gz;                             // sigma_z |grad depth| (k_s_variance)
    float4 *col, *tmp;
    kgk_camera pcam;
    int has_prev;
    int firefly;                           // clamp isolated samples before they enter the history
    float alpha, sz, sn, sl;
};

// Projects a world position into the previous camera (inverse of
// Generate1stRay): pixel coordinates (x, y) of the previous frame.
__device__ __forceinline__ bool project_prev(const kgk_camera &c, int W, int H, float3 p, float &x, float &y) {
    const float3 o = f3(c.CamOrg.x, c.CamOrg.y, c.CamOrg.z);
    const float3 d = f3(c.CamDir.x, c.CamDir.y, c.CamDir.z);
    const float3 sx = f3(c.ScreenXDir.x, c.ScreenXDir.y, c.ScreenXDir.z);
    const float3 sy = f3(c.ScreenYDir.x, c.ScreenYDir.y, c.ScreenYDir.z);
    const float3 v = p - o;
    const float z = dot3(v, d);
    if (z <= 1e-6f) return false;
    const float k = c.CamToScreenDist / z;  // scale to the screen plane
    x = dot3(v, sx) * k / (c.PixelSize * dot3(sx, sx)) + W / 2.0f;
    y = H / 2.0f - dot3(v, sy) * k / (c.PixelSize * dot3(sy, sy));
    return true;
}

constexpr float kFirefly = 4.0f;

// Temporal integration; also writes this frame's guide (normal + depth,
// material id) that the spatial passes read and the next frame reprojects
// against.
__global__ void k_s_temporal(StdArgs a) {
    const int W = a.W, H = a.H;
    FOR_PIXELS(W * H) {
        const float4 nr = a.nrm[p];
        const int obj = __float_as_int(nr.w);
        const float3 noisy = f3(a.noisy[p]);
        const float4 ps = a.pos[p];
        if (obj < 0) {
            a.hist[p] = make_float4(noisy.x, noisy.y, noisy.z, 0.0f);
            a.mom[p] = make_float2(0.0f, 0.0f);
            a.col[p] = make_float4(noisy.x, noisy.y, noisy.z, 0.0f);
            a.nd[p] = make_float4(nr.x, nr.y, nr.z, ps.w);
            a.mat[p] = -1;
            continue;
        }
        const float4 al = a.alb[p];
        const int mat = max(__float_as_int(al.w), 0);
        a.nd[p] = make_float4(nr.x, nr.y, nr.z, ps.w);
        a.mat[p] = mat;
        const float3 albedo = f3(al);
        float3 dl = div3(noisy, albedo + f3(kS, kS, kS));
        float l = lumf(dl);
        // temporal mode: the colour box of the 3 x 3 neighbourhood (pixels
        // that hit) that the reprojected history is clamped to
        float3 bmin = f3(0.0f, 0.0f, 0.0f), bmax = f3(0.0f, 0.0f, 0.0f);
        if (a.firefly) {
            // an isolated sample more than kFirefly times as bright as the
            // brightest of its eight neighbours (that hit) is scaled down to
            // that bound before it enters the history, where alpha = 0.2
            // would carry it for tens of frames
            const int x = p % W, y = p / W;
            float lmax = 0.0f;
            bool any = false;
            bmin = f3(3.0e38f, 3.0e38f, 3.0e38f);
            bmax = f3(-3.0e38f, -3.0e38f, -3.0e38f);
            for (int k = 0; k < 9; ++k) {
                const int qx = x + k % 3 - 1, qy = y + k / 3 - 1;
                if (k == 4 || qx < 0 || qx >= W || qy < 0 || qy >= H) continue;
                const int q = W * qy + qx;
                if (__float_as_int(a.nrm[q].w) < 0) continue;
                any = true;
                const float3 dq = div3(f3(a.noisy[q]), f3(a.alb[q]) + f3(kS, kS, kS));
                lmax = fmaxf(lmax, lumf(dq));
                bmin = f3(fminf(bmin.x, dq.x), fminf(bmin.y, dq.y), fminf(bmin.z, dq.z));
                bmax = f3(fmaxf(bmax.x, dq.x), fmaxf(bmax.y, dq.y), fmaxf(bmax.z, dq.z));
            }
            const float cap = kFirefly * lmax + 1e-3f;
            if (any && l > cap) {
                dl = dl * (cap / l);
                l = cap;
            }
            bmin = f3(fminf(bmin.x, dl.x), fminf(bmin.y, dl.y), fminf(bmin.z, dl.z));
            bmax = f3(fmaxf(bmax.x, dl.x), fmaxf(bmax.y, dl.y), fmaxf(bmax.z, dl.z));
        }
        float3 hc = f3(0.0f, 0.0f, 0.0f);
        float2 hm = make_float2(0.0f, 0.0f);
        float hl = 0.0f, wsum = 0.0f;
        if (a.has_prev) {
            float x, y;
            if (project_prev(a.pcam, W, H, f3(ps), x, y)) {
                // bilinear taps; pixel (X, Y)'s primary ray passes through
                // integer screen coordinates (Generate1stRay)
                const float fx = x, fy = y;
                const int x0 = (int)floorf(fx), y0 = (int)floorf(fy);
                const float tx = fx - x0, ty = fy - y0;
                const float3 pc = f3(a.pcam.CamOrg.x, a.pcam.CamOrg.y, a.pcam.CamOrg.z);
                const float exp_depth = len3(f3(ps) - pc);
                for (int k = 0; k < 4; ++k) {
                    const int qx = x0 + (k & 1), qy = y0 + (k >> 1);
                    if (qx < 0 || qx >= W || qy < 0 || qy >= H) continue;
                    const int q = W * qy + qx;
                    if (a.mat_prev[q] != mat) continue;
                    const float4 pn = a.nd_prev[q];
                    if (dot3(f3(pn), f3(nr)) < 0.9f) continue;
                    if (fabsf(pn.w - exp_depth) > 0.05f * exp_depth + 1e-3f) continue;
                    const float w = ((k & 1) ? tx : 1.0f - tx) * ((k >> 1) ? ty : 1.0f - ty);
                    const float4 hp = a.hist_prev[q];
                    const float2 mp = a.mom_prev[q];
                    hc += f3(hp) * w;
                    hl += hp.w * w;
                    hm.x += mp.x * w;
                    hm.y += mp.y * w;
                    wsum += w;
                }
            }
        }
        float3 c;
        float2 m;
        float len;
        if (wsum > 1e-4f) {
            hc = hc / wsum;
            if (a.firefly)  // history outside the current neighbourhood's box is stale (ghosting)
                hc = f3(fminf(fmaxf(hc.x, bmin.x), bmax.x), fminf(fmaxf(hc.y, bmin.y), bmax.y),
                        fminf(fmaxf(hc.z, bmin.z), bmax.z));
            hm.x /= wsum;
            hm.y /= wsum;
            len = fminf(hl / wsum + 1.0f, 64.0f);
            const float ac = fmaxf(a.alpha, 1.0f / len);
            c = hc * (1.0f - ac) + dl * ac;
            m = make_float2(hm.x * (1.0f - ac) + l * ac, hm.y * (1.0f - ac) + l * l * ac);
        } else {
            c = dl;
            m = make_float2(l, l * l);
            len = 1.0f;
        }
        a.hist[p] = make_float4(c.x, c.y, c.z, len);
        a.mom[p] = m;
        a.col[p] = make_float4(c.x, c.y, c.z, 0.0f);
    }
}

// The spatial passes' edge-stopping weight is one base-2 exponential:
//   w = max(0, n.nq)^sigma_n * exp(-|d - dq| / (sigma_z |grad d| dist + 1e-3))
//                            * exp(-|l - lq| / (sigma_l sqrt(var) + 1e-6))
//     = 2^(sigma_n log2 max(0, n.nq) - |d - dq| rz(dist) - |l - lq| rl)
// with rz(dist) = log2(e) / (sigma_z |grad d| dist + 1e-3) taken once per
// pixel for each distinct tap distance, and rl likewise; lg2(0) = -inf gives
// w = 0 for normals facing away.  Both are the hardware approximations
// (ex2.approx / lg2.approx, relative error ~2^-22).
constexpr float kLog2e = 1.44269504088896341f;
__device__ __forceinline__ float ex2a(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float lg2a(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Tiles of the standard filter's spatial passes: 32 x 8 pixels and a halo of
// R pixels.  Entries outside the image carry material -2, which matches no
// pixel, so taps need no bounds test.
constexpr int kSTX = 32, kSTY = 8;

// Variance: temporal moments when the history is long enough (>= 4 frames),
// else a 7 x 7 edge-stopped spatial estimate (normal and depth weights) on a
// shared-memory tile with a halo of 3.
__global__ void __launch_bounds__(256) k_s_variance(StdArgs a) {
    constexpr int R = 3, SX = kSTX + 2 * R, SY = kSTY + 2 * R;
    __shared__ float4 s_nd[SY * SX];
    __shared__ float2 s_mo[SY * SX];
    __shared__ int s_m[SY * SX];
    const int W = a.W, H = a.H;
    const int x0 = blockIdx.x * kSTX - R, y0 = blockIdx.y * kSTY - R;
    for (int i = threadIdx.y * kSTX + threadIdx.x; i < SX * SY; i += kSTX * kSTY) {
        const int gx = x0 + i % SX, gy = y0 + i / SX;
        if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
            const int q = W * gy + gx;
            s_nd[i] = a.nd[q];
            s_mo[i] = a.mom[q];
            s_m[i] = a.mat[q];
        } else {
            s_m[i] = -2;
        }
    }
    __syncthreads();
    const int x = blockIdx.x * kSTX + threadIdx.x, y = blockIdx.y * kSTY + threadIdx.y;
    if (x >= W || y >= H) return;
    const int p = W * y + x, c = SX * (threadIdx.y + R) + threadIdx.x + R;
    const int mat = s_m[c];
    if (mat < 0) return;
    // sigma_z |grad d|: central differences of the depth (one-sided at the
    // border), kept for the a-trous passes
    const float4 nd = s_nd[c];
    const float d = nd.w;
    const float gx = (x + 1 < W ? s_nd[c + 1].w : d) - (x > 0 ? s_nd[c - 1].w : d);
    const float gy = (y + 1 < H ? s_nd[c + SX].w : d) - (y > 0 ? s_nd[c - SX].w : d);
    const float kz = a.sz * 0.5f * fmaxf(fabsf(gx), fabsf(gy));
    a.gz[p] = kz;
    const float len = a.hist[p].w;
    float var;
    if (len >= 4.0f) {
        const float2 m = s_mo[c];
        var = fmaxf(0.0f, m.y - m.x * m.x);
    } else {
        // rz for the 10 distinct squared distances of a 7 x 7 window
        constexpr int kD2[10] = {0, 1, 2, 4, 5, 8, 9, 10, 13, 18};
        float rz[10];
#pragma unroll
        for (int k = 0; k < 10; ++k) rz[k] = kLog2e / (kz * sqrtf((float)kD2[k]) + 1e-3f);
        float s1 = 0, s2 = 0, sw = 0;
#pragma unroll
        for (int ky = -3; ky <= 3; ++ky)
#pragma unroll
            for (int kx = -3; kx <= 3; ++kx) {
                const int t = c + SX * ky + kx;
                if (s_m[t] != mat) continue;
                const int d2 = kx * kx + ky * ky;
                const int cls = d2 == 0 ? 0 : d2 == 1 ? 1 : d2 == 2 ? 2 : d2 == 4 ? 3 : d2 == 5 ? 4 : d2 == 8 ? 5
                              : d2 == 9 ? 6 : d2 == 10 ? 7 : d2 == 13 ? 8 : 9;
                const float4 qn = s_nd[t];
                const float e = a.sn * lg2a(fmaxf(0.0f, dot3(f3(nd), f3(qn)))) - fabsf(d - qn.w) * rz[cls];
                const float w = ex2a(e);
                const float2 m = s_mo[t];
                s1 += w * m.x;
                s2 += w * m.y;
                sw += w;
            }
        var = sw > 0.0f ? fmaxf(0.0f, s2 / sw - (s1 / sw) * (s1 / sw)) : 0.0f;
        var *= 4.0f / len;  // boost for short histories
    }
    a.col[p].w = var;
}

// k_s_gauss_var's 3 x 3 blur of the variance over the pixels in the image,
// read from global memory around pixel p = (x, y).
__device__ __forceinline__ float gauss_var_global(const float4 *__restrict__ in, int W, int H, int x, int y) {
    float gs = 0, gw = 0;
#pragma unroll
    for (int ky = -1; ky <= 1; ++ky)
#pragma unroll
        for (int kx = -1; kx <= 1; ++kx) {
            if (x + kx < 0 || x + kx >= W || y + ky < 0 || y + ky >= H) continue;
            const float k = cKG[kx + 1] * cKG[ky + 1];
            gs += k * in[W * (y + ky) + x + kx].w;
            gw += k;
        }
    return gs / gw;
}

// One a-trous pass of pixel p at `step` over colour + variance, given the
// 3 x 3-blurred variance gvar.  Reads go through Src: a shared-memory tile
// (k_s_atrous_tile), staged rows (k_s_atrous_rows) or the global arrays
// (k_s_atrous).
template <class Src>
__device__ __forceinline__ float4 std_atrous_px(const StdArgs &a, const Src &S, int p, int step, float gvar) {
    const float4 c = S.c(0, 0);
    const int mat = S.m(0, 0);
    const float4 nd = S.nd(0, 0);
    const float d = nd.w;
    const float kz = a.gz[p] * (float)step;
    const float l = lumf(f3(c));
    const float rl = kLog2e / (a.sl * sqrtf(fmaxf(gvar, 0.0f)) + 1e-6f);
    // rz for the squared tap distances 1, 2, 4, 5, 8 (in steps)
    float rz[5];
    constexpr int kD2[5] = {1, 2, 4, 5, 8};
#pragma unroll
    for (int k = 0; k < 5; ++k) rz[k] = kLog2e / (kz * sqrtf((float)kD2[k]) + 1e-3f);
    float3 sc = f3(c) * (36.0f / 256.0f);
    float sv = (36.0f / 256.0f) * (36.0f / 256.0f) * c.w;
    float sw = 36.0f / 256.0f;
#pragma unroll
    for (int ki = 0; ki < 25; ++ki) {
        if (ki == 12) continue;
        const int ox = (ki % 5 - 2) * step, oy = (ki / 5 - 2) * step;
        if (!S.inside(ox, oy)) continue;
        if (S.m(ox, oy) != mat) continue;  // no hit, another material, or outside a tile's image
        const float4 qn = S.nd(ox, oy);
        const float4 qc = S.c(ox, oy);
        const int d2 = (ki % 5 - 2) * (ki % 5 - 2) + (ki / 5 - 2) * (ki / 5 - 2);
        const int cls = d2 == 1 ? 0 : d2 == 2 ? 1 : d2 == 4 ? 2 : d2 == 5 ? 3 : 4;
        const float e = a.sn * lg2a(fmaxf(0.0f, dot3(f3(nd), f3(qn)))) - fabsf(d - qn.w) * rz[cls] -
                        fabsf(l - lumf(f3(qc))) * rl;
        const float w = cKW[ki] * ex2a(e);
        sc += f3(qc) * w;
        sv += w * w * qc.w;
        sw += w;
    }
    return make_float4(sc.x / sw, sc.y / sw, sc.z / sw, sv / (sw * sw));
}

// The small steps (1, 2, 4) on shared-memory tiles with a halo of 2 * step:
// guide (normal, depth), material and colour + variance.  The first pass
// (kFeedback) also writes its colour back into the history, which the next
// frame integrates.
template <int kStep, bool kFeedback>
__global__ void __launch_bounds__(256) k_s_atrous_tile(StdArgs a, const float4 *__restrict__ in, float4 *out) {
    constexpr int R = 2 * kStep, SX = kSTX + 2 * R, SY = kSTY + 2 * R;
    __shared__ float4 s_nd[SY * SX];
    __shared__ float4 s_c[SY * SX];
    __shared__ int s_m[SY * SX];
    const int W = a.W, H = a.H;
    const int x0 = blockIdx.x * kSTX - R, y0 = blockIdx.y * kSTY - R;
    for (int i = threadIdx.y * kSTX + threadIdx.x; i < SX * SY; i += kSTX * kSTY) {
        const int gx = x0 + i % SX, gy = y0 + i / SX;
        if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
            const int q = W * gy + gx;
            s_nd[i] = a.nd[q];
            s_c[i] = in[q];
            s_m[i] = a.mat[q];
        } else {
            s_m[i] = -2;
        }
    }
    __syncthreads();
    const int x = blockIdx.x * kSTX + threadIdx.x, y = blockIdx.y * kSTY + threadIdx.y;
    if (x >= W || y >= H) return;
    struct {
        const float4 *snd, *sc;
        const int *sm;
        int o;  // this pixel's entry
        __device__ bool inside(int ox, int oy) const { return sm[o + SX * oy + ox] != -2; }
        __device__ int m(int ox, int oy) const { return sm[o + SX * oy + ox]; }
        __device__ float4 nd(int ox, int oy) const { return snd[o + SX * oy + ox]; }
        __device__ float4 c(int ox, int oy) const { return sc[o + SX * oy + ox]; }
    } S{s_nd, s_c, s_m, SX * ((int)threadIdx.y + R) + (int)threadIdx.x + R};
    const int p = W * y + x;
    if (s_m[S.o] < 0) {
        out[p] = s_c[S.o];
        return;
    }
    // k_s_gauss_var's 3 x 3 blur of the variance over the pixels in the image
    float gs = 0, gw = 0;
#pragma unroll
    for (int ky = -1; ky <= 1; ++ky)
#pragma unroll
        for (int kx = -1; kx <= 1; ++kx) {
            if (!S.inside(kx, ky)) continue;
            const float k = cKG[kx + 1] * cKG[ky + 1];
            gs += k * S.c(kx, ky).w;
            gw += k;
        }
    const float4 o = std_atrous_px(a, S, p, kStep, gs / gw);
    out[p] = o;
    if (kFeedback) {
        const float len = a.hist[p].w;
        a.hist[p] = make_float4(o.x, o.y, o.z, len);
    }
}

// The large steps (8 and 16) on row segments: a block of 256 threads takes
// 256 pixels of one row and stages the five rows its taps read (y + {-2, -1,
// 0, 1, 2} step, 256 + 4 step entries each); the variance blur's neighbours
// come from global memory (coalesced: consecutive threads, consecutive
// pixels).
template <int kStep> struct SRows {
    static constexpr int T = 256, R = 2 * kStep, SX = T + 2 * R, N = 5 * SX;
    static constexpr size_t kSmem = (size_t)N * (2 * sizeof(float4) + sizeof(int));
};

template <int kStep>
__global__ void __launch_bounds__(256) k_s_atrous_rows(StdArgs a, const float4 *__restrict__ in, float4 *out) {
    using T = SRows<kStep>;
    extern __shared__ __align__(16) unsigned char smem[];
    float4 *s_nd = (float4 *)smem;
    float4 *s_c = s_nd + T::N;
    int *s_m = (int *)(s_c + T::N);
    const int W = a.W, H = a.H, y = blockIdx.y;
    const int x0 = blockIdx.x * T::T - T::R;
    for (int i = threadIdx.x; i < T::N; i += T::T) {
        const int gx = x0 + i % T::SX, gy = y + (i / T::SX - 2) * kStep;
        if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
            const int q = W * gy + gx;
            s_nd[i] = a.nd[q];
            s_c[i] = in[q];
            s_m[i] = a.mat[q];
        } else {
            s_m[i] = -2;
        }
    }
    __syncthreads();
    const int x = blockIdx.x * T::T + threadIdx.x;
    if (x >= W) return;
    struct {
        const float4 *snd, *sc;
        const int *sm;
        int o;  // this pixel's entry
        __device__ int at(int ox, int oy) const { return o + T::SX * (oy / kStep) + ox; }
        __device__ bool inside(int ox, int oy) const { return sm[at(ox, oy)] != -2; }
        __device__ int m(int ox, int oy) const { return sm[at(ox, oy)]; }
        __device__ float4 nd(int ox, int oy) const { return snd[at(ox, oy)]; }
        __device__ float4 c(int ox, int oy) const { return sc[at(ox, oy)]; }
    } S{s_nd, s_c, s_m, 2 * T::SX + (int)threadIdx.x + T::R};
    const int p = W * y + x;
    if (s_m[S.o] < 0) {
        out[p] = s_c[S.o];
        return;
    }
    out[p] = std_atrous_px(a, S, p, kStep, gauss_var_global(in, W, H, x, y));
}

// Steps of 32 and more (more than five a-trous passes): taps read global
// memory (through L1 and L2).  kStep = 0: the step is `step`.
template <int kStep>
__global__ void k_s_atrous(StdArgs a, const float4 *__restrict__ in, float4 *out, int step) {
    const int W = a.W, H = a.H;
    FOR_PIXELS(W * H) {
        const int x = p % W, y = p / W;
        struct {
            const float4 *gnd, *gc;
            const int *gm;
            int p, x, y, W, H;
            __device__ bool inside(int ox, int oy) const {
                return x + ox >= 0 && x + ox < W && y + oy >= 0 && y + oy < H;
            }
            __device__ int m(int ox, int oy) const { return gm[p + W * oy + ox]; }
            __device__ float4 nd(int ox, int oy) const { return gnd[p + W * oy + ox]; }
            __device__ float4 c(int ox, int oy) const { return gc[p + W * oy + ox]; }
        } S{a.nd, in, a.mat, p, x, y, W, H};
        if (a.mat[p] < 0) {
            out[p] = in[p];
            continue;
        }
        out[p] = std_atrous_px(a, S, p, kStep ? kStep : step, gauss_var_global(in, W, H, x, y));
    }
}

// The last pass: re-modulates the filtered colour by the albedo and writes
// the frame (out, when not null) and its save_png bytes (rgba8, when not null).
__global__ void k_s_output(StdArgs a, const float4 *filtered, float4 *out, uchar4 *rgba8,
                           const __grid_constant__ ToneTable T) {
    FOR_PIXELS(a.W * a.H) {
        const float4 c = filtered[p];
        float4 o;
        if (a.mat[p] < 0) {
            o = make_float4(c.x, c.y, c.z, 1.0f);
        } else {
            const float3 al = f3(a.alb[p]) + f3(kS, kS, kS);
            o = make_float4(c.x * al.x, c.y * al.y, c.z * al.z, 1.0f);
        }
        if (out) out[p] = o;
        if (rgba8) rgba8[p] = tone_rgba8(o, T);
    }
}

template <class T> kgk_status realloc_d(T **p, size_t n, const char *what) {
    dfree(*p);
    *p = nullptr;
    return dalloc(p, n, what);
}

}  // namespace

void svgf_state_free_impl(SvgfState *S) {
    void *ptrs[] = {S->prev, S->cur, S->hist, S->hist_prev, S->mom, S->mom_prev, S->nd, S->nd_prev,
                    S->mat, S->mat_prev, S->gz, S->col, S->tmp, S->compat_scratch};
    for (void *p : ptrs) dfree(p);
}

void svgf_state_free(kgk_scene *s) {
    if (!s->svgf) return;
    svgf_state_free_impl(s->svgf);
    delete s->svgf;
    s->svgf = nullptr;
}

SvgfState *svgf_state(kgk_scene *s) {
    if (!s->svgf) s->svgf = new SvgfState();
    return s->svgf;
}

kgk_status tonemap_device(const float4 *in, size_t npx, uchar4 *out, cudaStream_t st) {
    const int g = (int)std::min<size_t>((npx + 255) / 256, 4096);
    k_tonemap<<<g, 256, 0, st>>>(in, npx, out, tone_table());
    KGK_CUDA(cudaGetLastError());
    return KGK_OK;
}

void output_state_free(kgk_scene *s) {
    OutputState *O = s->out;
    if (!O) return;
    if (O->copy) cudaStreamSynchronize(O->copy);
    for (int k = 0; k < 2; ++k) {
        dfree(O->rgba8[k]);
        if (O->done[k]) cudaEventDestroy(O->done[k]);
        if (O->copied[k]) cudaEventDestroy(O->copied[k]);
    }
    if (O->copy) cudaStreamDestroy(O->copy);
    delete O;
    s->out = nullptr;
}

// The output double buffer for npx pixels (created on first use).
kgk_status output_state(kgk_scene *s, size_t npx, OutputState **out) {
    if (!s->out) {
        OutputState *O = new OutputState();
        s->out = O;
        KGK_CUDA(cudaStreamCreateWithFlags(&O->copy, cudaStreamNonBlocking));
        for (int k = 0; k < 2; ++k) {
            KGK_CUDA(cudaEventCreateWithFlags(&O->done[k], cudaEventDisableTiming));
            KGK_CUDA(cudaEventCreateWithFlags(&O->copied[k], cudaEventDisableTiming));
        }
    }
    OutputState &O = *s->out;
    if (O.npx < npx) {
        KGK_CUDA(cudaStreamSynchronize(O.copy));
        for (int k = 0; k < 2; ++k) {
            dfree(O.rgba8[k]);
            O.rgba8[k] = nullptr;
        }
        O.npx = 0;
        for (int k = 0; k < 2; ++k) KGK_TRY(dalloc(&O.rgba8[k], npx, "RGBA8 output"));
        O.npx = npx;
    }
    *out = &O;
    return KGK_OK;
}

}  // namespace kgk

using namespace kgk;

extern "C" {

kgk_status kgk_svgf_apply(kgk_vec *result, kgk_vec *filtered, kgk_svgf_buffer *prev, kgk_svgf_buffer *cur,
                          int32_t W, int32_t H, int32_t frame) {
    if (!result || !filtered || !prev || !cur) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_svgf_apply: NULL buffer");
    if (W < 2 || H < 2 || (long long)W * H > (1LL << 26))
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_svgf_apply: image size out of range (needs >= 2 x 2)");
    int dev = 0;
    KGK_CUDA(cudaGetDevice(&dev));
    cudaStream_t st;
    KGK_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const size_t npx = (size_t)W * H;
    const bool dr = is_device_ptr(result), df = is_device_ptr(filtered), dp = is_device_ptr(prev),
               dc = is_device_ptr(cur);
    kgk_vec *R = result, *F = filtered;
    kgk_svgf_buffer *P = prev, *C = cur;
    std::vector<void *> owned;
    auto stage = [&](void **dst, void *src, size_t bytes, bool is_dev) -> kgk_status {
        if (is_dev) { *dst = src; return KGK_OK; }
        KGK_TRY(dmalloc(dst, bytes, "SVGF staging"));
        owned.push_back(*dst);
        KGK_CUDA(cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, st));
        return KGK_OK;
    };
    kgk_status s = KGK_OK;
    if (s == KGK_OK) s = stage((void **)&R, result, npx * sizeof(kgk_vec), dr);
    if (s == KGK_OK) s = stage((void **)&F, filtered, npx * sizeof(kgk_vec), df);
    if (s == KGK_OK) s = stage((void **)&P, prev, npx * sizeof(kgk_svgf_buffer), dp);
    if (s == KGK_OK) s = stage((void **)&C, cur, npx * sizeof(kgk_svgf_buffer), dc);
    if (s == KGK_OK) s = run_compat(R, F, P, C, W, H, frame, 5, 5, st);
    if (s == KGK_OK) {
        cudaError_t e = cudaSuccess;
        if (!dr) e = cudaMemcpyAsync(result, R, npx * sizeof(kgk_vec), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && !df) e = cudaMemcpyAsync(filtered, F, npx * sizeof(kgk_vec), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && !dp) e = cudaMemcpyAsync(prev, P, npx * sizeof(kgk_svgf_buffer), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && !dc) e = cudaMemcpyAsync(cur, C, npx * sizeof(kgk_svgf_buffer), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) s = cuda_fail(e, "kgk_svgf_apply copies");
    }
    for (void *p : owned) dfree(p);
    cudaStreamDestroy(st);
    return s;
}

kgk_status kgk_gbuffer_records(kgk_scene *s, kgk_svgf_buffer *out) {
    if (!s || !out) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_gbuffer_records: NULL argument");
    KGK_CUDA(cudaSetDevice(s->device));
    int W, H;
    const float4 *gpos, *gnrm, *galb, *gemi;
    kgk_camera cam;
    if (!svgf_gbuffer(s, &W, &H, &gpos, &gnrm, &galb, &gemi, &cam))
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_gbuffer_records: render a frame with write_gbuffer=1 first");
    const size_t npx = (size_t)W * H;
    cudaStream_t st = s->stream;
    const bool dev = is_device_ptr(out);
    kgk_svgf_buffer *dst = out;
    if (!dev) {
        KGK_TRY(s->staging.reserve(npx * sizeof(kgk_svgf_buffer)));
        dst = (kgk_svgf_buffer *)s->staging.ptr;
    }
    k_gbuffer_to_records<<<(unsigned)((npx + 255) / 256), 256, 0, st>>>(gpos, gnrm, galb, gemi, npx, dst);
    KGK_CUDA(cudaGetLastError());
    if (!dev) KGK_CUDA(cudaMemcpyAsync(out, dst, npx * sizeof(kgk_svgf_buffer), cudaMemcpyDeviceToHost, st));
    KGK_CUDA(cudaStreamSynchronize(st));
    return KGK_OK;
}

kgk_status kgk_svgf(kgk_scene *s, const kgk_svgf_config *cfg, const kgk_vec *noisy, kgk_vec *filtered) {
    if (!s || !cfg || !noisy || !filtered) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_svgf: NULL argument");
    return kgk_svgf_output(s, cfg, noisy, filtered, nullptr, 0);
}

kgk_status kgk_svgf_output(kgk_scene *s, const kgk_svgf_config *cfg, const kgk_vec *noisy, kgk_vec *filtered,
                           uint8_t *rgba8, int32_t async) {
    if (!s || !cfg) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_svgf: NULL argument");
    if (!filtered && !rgba8) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_svgf: no output buffer");
    KGK_CUDA(cudaSetDevice(s->device));
    int W, H;
    const float4 *gpos, *gnrm, *galb, *gemi;
    kgk_camera cam;
    if (!svgf_gbuffer(s, &W, &H, &gpos, &gnrm, &galb, &gemi, &cam))
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_svgf: render a frame with write_gbuffer=1 first");
    if (cfg->width != W || cfg->height != H)
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_svgf: size differs from the last rendered G-buffer");
    if (W < 2 || H < 2) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_svgf: image must be at least 2 x 2");
    SvgfState &S = *svgf_state(s);
    const size_t npx = (size_t)W * H;
    cudaStream_t st = s->stream;
    if (S.W != W || S.H != H) {
        svgf_state_free_impl(&S);
        S = SvgfState();
        KGK_TRY(dalloc(&S.prev, npx, "SVGF history"));
        KGK_TRY(dalloc(&S.cur, npx, "SVGF state"));
        KGK_TRY(dalloc(&S.hist, npx, "SVGF history"));
        KGK_TRY(dalloc(&S.hist_prev, npx, "SVGF history"));
        KGK_TRY(dalloc(&S.mom, npx, "SVGF moments"));
        KGK_TRY(dalloc(&S.mom_prev, npx, "SVGF moments"));
        KGK_TRY(dalloc(&S.nd, npx, "SVGF guide"));
        KGK_TRY(dalloc(&S.nd_prev, npx, "SVGF history"));
        KGK_TRY(dalloc(&S.mat, npx, "SVGF guide"));
        KGK_TRY(dalloc(&S.mat_prev, npx, "SVGF history"));
        KGK_TRY(dalloc(&S.gz, npx, "SVGF guide"));
        KGK_TRY(dalloc(&S.col, npx, "SVGF colour"));
        KGK_TRY(dalloc(&S.tmp, npx, "SVGF colour"));
        KGK_TRY(dalloc(&S.compat_scratch, compat_scratch_bytes(npx), "SVGF scratch"));
        KGK_CUDA(cudaMemset(S.prev, 0, npx * sizeof(kgk_svgf_buffer)));
        S.W = W;
        S.H = H;
        S.has_prev = false;
    }
    // input: the frame kept on the device by kgk_render(out = NULL), a device
    // image, or a host image staged here
    const float4 *kept = nullptr;
    if (!noisy) {
        int kW = 0, kH = 0;
        if (!render_kept_frame(s, &kW, &kH, &kept) || kW != W || kH != H)
            return fail(KGK_ERR_INVALID_ARGUMENT,
                        "kgk_svgf: noisy == NULL needs the last kgk_render to keep its frame (out == NULL)");
    }
    const bool dn = noisy && is_device_ptr(noisy), dfo = filtered && is_device_ptr(filtered);
    KGK_TRY(s->staging.reserve(2 * npx * sizeof(float4) + 256));
    float4 *in = kept ? (float4 *)kept : (dn ? (float4 *)noisy : (float4 *)s->staging.ptr);
    // the filtered frame: the caller's device buffer, else staging (copied to a
    // host buffer below, or only tone-mapped)
    float4 *out = dfo ? (float4 *)filtered : (float4 *)((char *)s->staging.ptr + npx * sizeof(float4));
    if (noisy && !dn) KGK_CUDA(cudaMemcpyAsync(in, noisy, npx * sizeof(float4), cudaMemcpyHostToDevice, st));
    // RGBA8 output: the caller's device buffer, else this scene's double buffer
    const bool d8 = rgba8 && is_device_ptr(rgba8);
    OutputState *O = nullptr;
    uchar4 *out8 = nullptr;
    int slot = 0;
    if (rgba8) {
        if (d8) {
            out8 = reinterpret_cast<uchar4 *>(rgba8);
        } else {
            KGK_TRY(output_state(s, npx, &O));
            slot = O->slot;
            O->slot ^= 1;
            out8 = O->rgba8[slot];
            // the copy that last read this buffer has finished
            KGK_CUDA(cudaStreamWaitEvent(st, O->copied[slot], 0));
        }
    }
    const int g = (int)std::min<size_t>((npx + 255) / 256, 65535);
    if (cfg->mode == KGK_SVGF_COMPAT) {
        k_gbuffer_to_records<<<(unsigned)((npx + 255) / 256), 256, 0, st>>>(gpos, gnrm, galb, gemi, npx, S.cur);
        // result buffer: the noisy frame (copied, the reference rewrites it)
        float4 *R = S.col;
        KGK_CUDA(cudaMemcpyAsync(R, in, npx * sizeof(float4), cudaMemcpyDeviceToDevice, st));
        const int reps = cfg->atrous_repeats > 0 ? cfg->atrous_repeats : 5;
        const int stages = cfg->atrous_iterations > 0 ? cfg->atrous_iterations : 5;
        KGK_TRY(run_compat((kgk_vec *)R, (kgk_vec *)out, S.prev, S.cur, W, H, cfg->frame_index, reps, stages, st,
                           S.compat_scratch));
        // main.cu:232: the current buffer becomes the previous one
        KGK_CUDA(cudaMemcpyAsync(S.prev, S.cur, npx * sizeof(kgk_svgf_buffer), cudaMemcpyDeviceToDevice, st));
        if (out8) KGK_TRY(tonemap_device(out, npx, out8, st));
    } else if (cfg->mode == KGK_SVGF_STANDARD || cfg->mode == KGK_SVGF_TEMPORAL) {
        if (cfg->frame_index == 0) S.has_prev = false;
        StdArgs a;
        a.W = W; a.H = H; a.pos = gpos; a.nrm = gnrm; a.alb = galb; a.emi = gemi; a.noisy = in;
        a.hist = S.hist; a.hist_prev = S.hist_prev; a.mom = S.mom; a.mom_prev = S.mom_prev;
        a.nd = S.nd; a.nd_prev = S.nd_prev; a.mat = S.mat; a.mat_prev = S.mat_prev;
        a.gz = S.gz; a.col = S.col; a.tmp = S.tmp;
        a.pcam = S.prev_cam;
        a.has_prev = S.has_prev ? 1 : 0;
        a.firefly = cfg->mode == KGK_SVGF_TEMPORAL ? 1 : 0;
        a.alpha = cfg->alpha > 0.0f ? cfg->alpha : 0.2f;
        a.sz = cfg->sigma_z > 0.0f ? cfg->sigma_z : 1.0f;
        a.sn = cfg->sigma_n > 0.0f ? cfg->sigma_n : 128.0f;
        a.sl = cfg->sigma_l > 0.0f ? cfg->sigma_l : 4.0f;
        const dim3 tiles((W + kSTX - 1) / kSTX, (H + kSTY - 1) / kSTY), tile_threads(kSTX, kSTY);
        const dim3 rows((W + 255) / 256, H);
        KGK_CUDA(cudaFuncSetAttribute(k_s_atrous_rows<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)SRows<8>::kSmem));
        KGK_CUDA(cudaFuncSetAttribute(k_s_atrous_rows<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)SRows<16>::kSmem));
        k_s_temporal<<<g, 256, 0, st>>>(a);
        const int iters = cfg->mode == KGK_SVGF_TEMPORAL ? 0 : cfg->atrous_iterations > 0 ? cfg->atrous_iterations : 5;
        if (iters > 0) k_s_variance<<<tiles, tile_threads, 0, st>>>(a);
        float4 *src = S.col, *dst = S.tmp;
        for (int i = 0; i < iters; ++i) {
            switch (i) {
                case 0: k_s_atrous_tile<1, true><<<tiles, tile_threads, 0, st>>>(a, src, dst); break;
                case 1: k_s_atrous_tile<2, false><<<tiles, tile_threads, 0, st>>>(a, src, dst); break;
                case 2: k_s_atrous_tile<4, false><<<tiles, tile_threads, 0, st>>>(a, src, dst); break;
                case 3: k_s_atrous_rows<8><<<rows, 256, SRows<8>::kSmem, st>>>(a, src, dst); break;
                case 4: k_s_atrous_rows<16><<<rows, 256, SRows<16>::kSmem, st>>>(a, src, dst); break;
                default: k_s_atrous<0><<<g, 256, 0, st>>>(a, src, dst, 1 << std::min(i, 24)); break;
            }
            std::swap(src, dst);
        }
        k_s_output<<<g, 256, 0, st>>>(a, src, filtered ? out : nullptr, out8, tone_table());
        KGK_CUDA(cudaGetLastError());
        // this frame's guide is the next frame's previous one
        std::swap(S.nd, S.nd_prev);
        std::swap(S.mat, S.mat_prev);
        std::swap(S.hist, S.hist_prev);
        std::swap(S.mom, S.mom_prev);
        S.prev_cam = cam;
        S.has_prev = true;
    } else {
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_svgf: unknown mode");
    }
    if (O) {
        // bring the bytes back on the copy stream, after this frame's filter
        KGK_CUDA(cudaEventRecord(O->done[slot], st));
        KGK_CUDA(cudaStreamWaitEvent(O->copy, O->done[slot], 0));
        KGK_CUDA(cudaMemcpyAsync(rgba8, out8, npx * sizeof(uchar4), cudaMemcpyDeviceToHost, O->copy));
        KGK_CUDA(cudaEventRecord(O->copied[slot], O->copy));
        if (!async) KGK_CUDA(cudaStreamSynchronize(O->copy));
    }
    if (filtered && !dfo) KGK_CUDA(cudaMemcpyAsync(filtered, out, npx * sizeof(float4), cudaMemcpyDeviceToHost, st));
    if (!async || (filtered && !dfo)) KGK_CUDA(cudaStreamSynchronize(st));
    return KGK_OK;
}

kgk_status kgk_scene_sync(kgk_scene *s) {
    if (!s) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_scene_sync: NULL scene");
    KGK_CUDA(cudaSetDevice(s->device));
    KGK_CUDA(cudaStreamSynchronize(s->stream));
    if (s->out) KGK_CUDA(cudaStreamSynchronize(s->out->copy));
    return KGK_OK;
}

kgk_status kgk_host_alloc(size_t bytes, void **out) {
    if (!out) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_host_alloc: NULL argument");
    *out = nullptr;
    const cudaError_t e = cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocPortable);
    if (e != cudaSuccess) {
        *out = nullptr;
        return cuda_fail(e, "kgk_host_alloc");
    }
    return KGK_OK;
}

void kgk_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free ApplySVGF (kgk_svgf_apply_noalloc).
//
// Some callers cannot call cudaMalloc: applications that reserve all device
// memory for their own pool allocator at start-up, and per-frame loops that
// must not allocate because cudaMalloc / cudaFree synchronise the whole device
// and stall the caller's other streams.  This entry point takes its scratch
// from g_svgf_scratch, a file-scope device array sized for
// KGK_SVGF_NOALLOC_MAX_PIXELS pixels (129 B per pixel, ~34 MB); every GPU that
// loads the library holds that array until the process exits.
// ---------------------------------------------------------------------------
#include <mutex>

namespace kgk {
namespace {

constexpr size_t kNaMax = (size_t)KGK_SVGF_NOALLOC_MAX_PIXELS;
// run_compat's scratch layout at the maximum image size
constexpr size_t kNaBytes = compat_scratch_bytes(kNaMax);

__device__ __align__(256) static unsigned char g_svgf_scratch[kNaBytes];

constexpr int kNaMaxDevices = 64;
std::mutex g_na_mu;
unsigned char *g_na_addr[kNaMaxDevices] = {};

// Device address of g_svgf_scratch on the current device; looked up once per
// device (with that device current) and cached for the life of the process,
// so it is stale after cudaDeviceReset on that device.
kgk_status noalloc_scratch(unsigned char **out) {
    int dev = 0;
    KGK_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNaMaxDevices) return fail(KGK_ERR_NO_DEVICE, "kgk_svgf_apply_noalloc: device index too large");
    std::lock_guard<std::mutex> lock(g_na_mu);
    if (!g_na_addr[dev]) {
        unsigned char *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&ptr, g_svgf_scratch);
        if (e != cudaSuccess || !ptr) return cuda_fail(e, "cudaGetSymbolAddress(g_svgf_scratch)");
        g_na_addr[dev] = ptr;
    }
    *out = g_na_addr[dev];
    return KGK_OK;
}

}  // namespace
}  // namespace kgk

extern "C" kgk_status kgk_svgf_apply_noalloc(kgk_vec *result, kgk_vec *filtered, kgk_svgf_buffer *prev,
                                             kgk_svgf_buffer *cur, int32_t W, int32_t H, int32_t frame,
                                             void *cuda_stream) {
    using namespace kgk;
    if (!result || !filtered || !prev || !cur)
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_svgf_apply_noalloc: NULL buffer");
    if (W < 2 || H < 2) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_svgf_apply_noalloc: image must be at least 2 x 2");
    if ((long long)W * H > (long long)KGK_SVGF_NOALLOC_MAX_PIXELS)
        return fail(KGK_ERR_INVALID_ARGUMENT,
                    "kgk_svgf_apply_noalloc: " + std::to_string((long long)W * H) + " pixels exceed the maximum of " +
                        std::to_string(KGK_SVGF_NOALLOC_MAX_PIXELS) + " (use kgk_svgf_apply)");
    if (!is_device_ptr(result) || !is_device_ptr(filtered) || !is_device_ptr(prev) || !is_device_ptr(cur))
        return fail(KGK_ERR_INVALID_ARGUMENT,
                    "kgk_svgf_apply_noalloc: all four buffers must be device memory (host buffers would need staging)");
    unsigned char *base = nullptr;
    KGK_TRY(noalloc_scratch(&base));
    CompatArgs a;
    a.W = W; a.H = H; a.frame = frame;
    a.R = result; a.F = filtered; a.P = prev; a.C = cur;
    // run_compat's layout, each array at its size for the largest image
    float *var2 = carve_compat(a, base, compat_fl(kNaMax), compat_vec(kNaMax));
    return launch_compat(a, var2, 5, 5, (cudaStream_t)cuda_stream);
}
