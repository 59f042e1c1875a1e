// bvh.cu - GPU binned-SAH BVH build and collapse into 8-wide compressed
// nodes.  Replaces the host build construct_BVH / Divide_AABB
// (ConstructBVH.cuh:13-207) and the per-node cudaMalloc upload
// (struct_BVH_node.cuh:72-83).
//
// Pipeline (all on the device stream; the host only orders the launches):
//   1. primitive boxes + scene bounds;
//   2. large tasks (> kSmall primitives): one level at a time, many blocks per
//      task: 32-bin centroid binning per axis (shared-memory atomics merged
//      into per-task global bins), one warp evaluates SAH over the 3 x 31
//      planes, a chunked stable partition (block scans) reorders the refs;
//   3. small tasks (<= kSmall): one block builds the whole subtree in shared
//      memory, always descending into the smaller child so its stack stays
//      <= log2(kSmall) deep; node ids come from a per-task reserved range, so
//      the tree is deterministic;
//   4. collapse: a bottom-up pass fills the SAH cost table of the optimal
//      collapse (k_dp_up); then breadth first, every wide node takes the 8
//      children that table chose; children with at most 1 (large scenes) or 3
//      (small ones) triangles are leaf children; slots are ordered by octant so traversal visits near
//      children first; child boxes are quantised to 8 bits against the parent
//      box (conservative rounding).
// Every kernel bounds-checks its writes and raises an error flag instead of
// writing out of range.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "kgk_device.cuh"
#include "kgk_internal.h"

namespace kgk {
namespace {

constexpr int kBins = 32;
constexpr int kChunk = 4096;   // primitives per block in the large-task path
constexpr int kSmall = 2048;   // tasks up to this size build inside one block
// Triangles per leaf child of a wide node, chosen per scene (bvh_build).
// One for large scenes: a wide node's leaf children then hold a triangle
// each, so its quantised child box culls that triangle alone, and a node
// yields at most 8 triangle tests.  Measured on the C2 frame (5.2M
// triangles): 3089 Mrays/s at 1, 2978 at 2, 2799 at 3 (extend 43.5 / 46.0 /
// 50.3 ms), for 1.72M / 1.00M / 0.71M wide nodes and a 140 / 87 / 65 ms
// build.  Three for small scenes, whose nodes and triangles stay in cache:
// the 36-triangle Cornell box (C1) runs 1509 Mrays/s at 3, 1156 at 1.
constexpr int kMaxLeaf = 3;                // the largest leaf the node format holds (8 x 3 = 24 bits)
constexpr int kLeafLarge = 1;
constexpr int kLargeSceneTris = 1 << 16;   // scenes above this use kLeafLarge
constexpr int kThreads = 256;
constexpr int kBinInts = 13;   // count, box lo/hi, centroid lo/hi (ordered ints)
constexpr int kStack = 32;

enum BuildError : int {
    kErrNone = 0,
    kErrSmallTooBig = 1,
    kErrNodeOverflow = 2,
    kErrStackOverflow = 3,
    kErrWideOverflow = 4,
    kErrTriOverflow = 5,
    kErrBadChild = 6,
};

struct Task {
    int node, begin, count, pad;
    float clo[3], chi[3];
    float pad2[2];
};

struct Split {
    int axis;   // -1: split by position
    int bin;
    int nleft;
    int pad;
    float lo[2][3], hi[2][3];    // child boxes (0 = left, 1 = right)
    float clo[2][3], chi[2][3];  // child centroid bounds
};

__device__ __forceinline__ void raise_err(int *err, int code) { atomicCAS(err, 0, code); }

__device__ __forceinline__ int bin_of(float c, float lo, float scale) {
    int b = (int)((c - lo) * scale);
    return b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
}

// Bin scale of one axis: kBins / extent, 0 for a flat axis.
__device__ __forceinline__ float bin_scale(float lo, float hi) {
    float e = hi - lo;
    return e > 0.0f ? (float)kBins / e : 0.0f;
}

__device__ __forceinline__ float3 centroid(float4 lo, float4 hi) {
    return f3(0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z));
}

// ---------------------------------------------------------------------------
// 1. primitive boxes
// ---------------------------------------------------------------------------
__global__ void k_init_bounds(int *g) {
    int i = threadIdx.x;
    if (i < 12) g[i] = (i % 6) < 3 ? f2o(INFINITY) : f2o(-INFINITY);
}

__global__ void k_prim_bounds(const float4 *__restrict__ verts, int n, float4 *plo, float4 *phi,
                              int *ref, int *gbounds) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float3 lo = f3(INFINITY, INFINITY, INFINITY), hi = f3(-INFINITY, -INFINITY, -INFINITY);
    float3 clo = lo, chi = hi;
    if (i < n) {
        float3 a = f3(verts[3 * i]), b = f3(verts[3 * i + 1]), c = f3(verts[3 * i + 2]);
        lo = fmin3(a, fmin3(b, c));
        hi = fmax3(a, fmax3(b, c));
        plo[i] = f4(lo, 0.0f);
        phi[i] = f4(hi, 0.0f);
        ref[i] = i;
        clo = chi = f3(0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = fmin3(lo, f3(__shfl_xor_sync(~0u, lo.x, o), __shfl_xor_sync(~0u, lo.y, o), __shfl_xor_sync(~0u, lo.z, o)));
        hi = fmax3(hi, f3(__shfl_xor_sync(~0u, hi.x, o), __shfl_xor_sync(~0u, hi.y, o), __shfl_xor_sync(~0u, hi.z, o)));
        clo = fmin3(clo, f3(__shfl_xor_sync(~0u, clo.x, o), __shfl_xor_sync(~0u, clo.y, o), __shfl_xor_sync(~0u, clo.z, o)));
        chi = fmax3(chi, f3(__shfl_xor_sync(~0u, chi.x, o), __shfl_xor_sync(~0u, chi.y, o), __shfl_xor_sync(~0u, chi.z, o)));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&gbounds[0], f2o(lo.x)); atomicMin(&gbounds[1], f2o(lo.y)); atomicMin(&gbounds[2], f2o(lo.z));
        atomicMax(&gbounds[3], f2o(hi.x)); atomicMax(&gbounds[4], f2o(hi.y)); atomicMax(&gbounds[5], f2o(hi.z));
        atomicMin(&gbounds[6], f2o(clo.x)); atomicMin(&gbounds[7], f2o(clo.y)); atomicMin(&gbounds[8], f2o(clo.z));
        atomicMax(&gbounds[9], f2o(chi.x)); atomicMax(&gbounds[10], f2o(chi.y)); atomicMax(&gbounds[11], f2o(chi.z));
    }
}

// ---------------------------------------------------------------------------
// Split evaluation by one warp over bins[3][kBins][kBinInts].
// ---------------------------------------------------------------------------
struct WarpSplit {
    int axis, bin;
    float cost;
};

__device__ __forceinline__ float3 shfl_up3(float3 v, int o) {
    return f3(__shfl_up_sync(~0u, v.x, o), __shfl_up_sync(~0u, v.y, o), __shfl_up_sync(~0u, v.z, o));
}
__device__ __forceinline__ float3 shfl_down3(float3 v, int o) {
    return f3(__shfl_down_sync(~0u, v.x, o), __shfl_down_sync(~0u, v.y, o), __shfl_down_sync(~0u, v.z, o));
}

// Scans one axis: on return lane b holds left (bins 0..b) and right
// (bins b+1..31) counts/boxes/centroid boxes.
struct AxisScan {
    int lc, rc;
    float3 llo, lhi, rlo, rhi, lclo, lchi, rclo, rchi;
};

__device__ AxisScan scan_axis(const int *bins, int axis) {
    const int lane = threadIdx.x & 31;
    const int *B = bins + (axis * kBins + lane) * kBinInts;
    int cnt = B[0];
    float3 lo = f3(o2f(B[1]), o2f(B[2]), o2f(B[3])), hi = f3(o2f(B[4]), o2f(B[5]), o2f(B[6]));
    float3 clo = f3(o2f(B[7]), o2f(B[8]), o2f(B[9])), chi = f3(o2f(B[10]), o2f(B[11]), o2f(B[12]));
    int pc = cnt, sc = cnt;
    float3 plo = lo, phi = hi, pclo = clo, pchi = chi;
    float3 slo = lo, shi = hi, sclo = clo, schi = chi;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int a = __shfl_up_sync(~0u, pc, o);
        float3 alo = shfl_up3(plo, o), ahi = shfl_up3(phi, o), aclo = shfl_up3(pclo, o), achi = shfl_up3(pchi, o);
        int b = __shfl_down_sync(~0u, sc, o);
        float3 blo = shfl_down3(slo, o), bhi = shfl_down3(shi, o), bclo = shfl_down3(sclo, o), bchi = shfl_down3(schi, o);
        if (lane >= o) {
            pc += a; plo = fmin3(plo, alo); phi = fmax3(phi, ahi); pclo = fmin3(pclo, aclo); pchi = fmax3(pchi, achi);
        }
        if (lane + o < 32) {
            sc += b; slo = fmin3(slo, blo); shi = fmax3(shi, bhi); sclo = fmin3(sclo, bclo); schi = fmax3(schi, bchi);
        }
    }
    AxisScan r;
    r.lc = pc; r.llo = plo; r.lhi = phi; r.lclo = pclo; r.lchi = pchi;
    r.rc = __shfl_down_sync(~0u, sc, 1);
    r.rlo = shfl_down3(slo, 1); r.rhi = shfl_down3(shi, 1);
    r.rclo = shfl_down3(sclo, 1); r.rchi = shfl_down3(schi, 1);
    if (lane == 31) r.rc = 0;
    return r;
}

// Best plane over all axes (lowest cost, ties -> lowest axis, then lowest bin).
__device__ WarpSplit warp_best_split(const int *bins) {
    const int lane = threadIdx.x & 31;
    WarpSplit best{-1, -1, INFINITY};
    for (int a = 0; a < 3; ++a) {
        AxisScan s = scan_axis(bins, a);
        float cost = INFINITY;
        if (lane < 31 && s.lc > 0 && s.rc > 0)
            cost = surface_area(s.llo, s.lhi) * (float)s.lc + surface_area(s.rlo, s.rhi) * (float)s.rc;
        float c = cost;
        int l = lane;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            float c2 = __shfl_xor_sync(~0u, c, o);
            int l2 = __shfl_xor_sync(~0u, l, o);
            if (c2 < c || (c2 == c && l2 < l)) { c = c2; l = l2; }
        }
        if (c < best.cost) { best.cost = c; best.axis = a; best.bin = l; }
    }
    return best;
}

__device__ void init_bins(int *bins) {
    for (int i = threadIdx.x; i < 3 * kBins * kBinInts; i += blockDim.x) {
        int k = i % kBinInts;
        bins[i] = k == 0 ? 0 : ((k - 1) % 6 < 3 ? f2o(INFINITY) : f2o(-INFINITY));
    }
}

__device__ __forceinline__ void bin_prim(int *bins, float4 lo, float4 hi, float3 c, const float *clo,
                                         const float *sc, bool cbox) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int b = bin_of(comp(c, a), clo[a], sc[a]);
        int *B = bins + (a * kBins + b) * kBinInts;
        atomicAdd(&B[0], 1);
        atomicMin(&B[1], f2o(lo.x)); atomicMin(&B[2], f2o(lo.y)); atomicMin(&B[3], f2o(lo.z));
        atomicMax(&B[4], f2o(hi.x)); atomicMax(&B[5], f2o(hi.y)); atomicMax(&B[6], f2o(hi.z));
        if (cbox) {
            atomicMin(&B[7], f2o(c.x)); atomicMin(&B[8], f2o(c.y)); atomicMin(&B[9], f2o(c.z));
            atomicMax(&B[10], f2o(c.x)); atomicMax(&B[11], f2o(c.y)); atomicMax(&B[12], f2o(c.z));
        }
    }
}

// ---------------------------------------------------------------------------
// 2. large tasks
// ---------------------------------------------------------------------------
struct Chunk {
    int task, begin, end, pad;
};

__global__ void k_init_global_bins(int *gbins, int ntasks) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntasks * 3 * kBins * kBinInts) return;
    int k = i % kBinInts;
    gbins[i] = k == 0 ? 0 : ((k - 1) % 6 < 3 ? f2o(INFINITY) : f2o(-INFINITY));
}

__global__ void __launch_bounds__(kThreads) k_bin_large(const Chunk *chunks, const Task *tasks,
                                                        const int *ref, const float4 *plo,
                                                        const float4 *phi, int *gbins) {
    __shared__ int bins[3 * kBins * kBinInts];
    const Chunk ch = chunks[blockIdx.x];
    const Task tk = tasks[ch.task];
    float sc[3];
    for (int a = 0; a < 3; ++a) sc[a] = bin_scale(tk.clo[a], tk.chi[a]);
    init_bins(bins);
    __syncthreads();
    for (int i = ch.begin + threadIdx.x; i < ch.end; i += blockDim.x) {
        int p = ref[i];
        float4 lo = plo[p], hi = phi[p];
        bin_prim(bins, lo, hi, centroid(lo, hi), tk.clo, sc, true);
    }
    __syncthreads();
    int *G = gbins + (size_t)ch.task * 3 * kBins * kBinInts;
    for (int i = threadIdx.x; i < 3 * kBins; i += blockDim.x) {
        const int *B = bins + i * kBinInts;
        if (B[0] == 0) continue;
        int *D = G + i * kBinInts;
        atomicAdd(&D[0], B[0]);
        for (int k = 1; k <= 3; ++k) atomicMin(&D[k], B[k]);
        for (int k = 4; k <= 6; ++k) atomicMax(&D[k], B[k]);
        for (int k = 7; k <= 9; ++k) atomicMin(&D[k], B[k]);
        for (int k = 10; k <= 12; ++k) atomicMax(&D[k], B[k]);
    }
}

// One warp per task: SAH split and child boxes.
__global__ void k_split_large(const Task *tasks, int ntasks, const int *gbins, Split *out) {
    const int t = blockIdx.x;
    if (t >= ntasks) return;
    const int lane = threadIdx.x & 31;
    const int *bins = gbins + (size_t)t * 3 * kBins * kBinInts;
    WarpSplit best = warp_best_split(bins);
    Split s;
    memset(&s, 0, sizeof s);
    if (best.axis < 0) {
        // Every centroid in one bin on every axis: split by position, both
        // children conservatively take the parent's boxes.
        AxisScan a = scan_axis(bins, 0);
        // lane 31 holds the full box in its prefix
        float3 lo = f3(__shfl_sync(~0u, a.llo.x, 31), __shfl_sync(~0u, a.llo.y, 31), __shfl_sync(~0u, a.llo.z, 31));
        float3 hi = f3(__shfl_sync(~0u, a.lhi.x, 31), __shfl_sync(~0u, a.lhi.y, 31), __shfl_sync(~0u, a.lhi.z, 31));
        float3 clo = f3(__shfl_sync(~0u, a.lclo.x, 31), __shfl_sync(~0u, a.lclo.y, 31), __shfl_sync(~0u, a.lclo.z, 31));
        float3 chi = f3(__shfl_sync(~0u, a.lchi.x, 31), __shfl_sync(~0u, a.lchi.y, 31), __shfl_sync(~0u, a.lchi.z, 31));
        if (lane == 0) {
            s.axis = -1;
            s.bin = -1;
            s.nleft = tasks[t].count / 2;
            for (int c = 0; c < 2; ++c) {
                s.lo[c][0] = lo.x; s.lo[c][1] = lo.y; s.lo[c][2] = lo.z;
                s.hi[c][0] = hi.x; s.hi[c][1] = hi.y; s.hi[c][2] = hi.z;
                s.clo[c][0] = clo.x; s.clo[c][1] = clo.y; s.clo[c][2] = clo.z;
                s.chi[c][0] = chi.x; s.chi[c][1] = chi.y; s.chi[c][2] = chi.z;
            }
            out[t] = s;
        }
        return;
    }
    AxisScan a = scan_axis(bins, best.axis);
    if (lane == best.bin) {
        s.axis = best.axis;
        s.bin = best.bin;
        s.nleft = a.lc;
        s.lo[0][0] = a.llo.x; s.lo[0][1] = a.llo.y; s.lo[0][2] = a.llo.z;
        s.hi[0][0] = a.lhi.x; s.hi[0][1] = a.lhi.y; s.hi[0][2] = a.lhi.z;
        s.lo[1][0] = a.rlo.x; s.lo[1][1] = a.rlo.y; s.lo[1][2] = a.rlo.z;
        s.hi[1][0] = a.rhi.x; s.hi[1][1] = a.rhi.y; s.hi[1][2] = a.rhi.z;
        s.clo[0][0] = a.lclo.x; s.clo[0][1] = a.lclo.y; s.clo[0][2] = a.lclo.z;
        s.chi[0][0] = a.lchi.x; s.chi[0][1] = a.lchi.y; s.chi[0][2] = a.lchi.z;
        s.clo[1][0] = a.rclo.x; s.clo[1][1] = a.rclo.y; s.clo[1][2] = a.rclo.z;
        s.chi[1][0] = a.rchi.x; s.chi[1][1] = a.rchi.y; s.chi[1][2] = a.rchi.z;
        out[t] = s;
    }
}

__device__ __forceinline__ bool goes_left(const Task &tk, const Split &s, int pos, float3 c) {
    if (s.axis < 0) return pos - tk.begin < s.nleft;
    return bin_of(comp(c, s.axis), tk.clo[s.axis], bin_scale(tk.clo[s.axis], tk.chi[s.axis])) <= s.bin;
}

__global__ void __launch_bounds__(kThreads) k_part_count(const Chunk *chunks, const Task *tasks,
                                                         const Split *splits, const int *ref,
                                                         const float4 *plo, const float4 *phi,
                                                         int *chunk_left) {
    __shared__ int red;
    const Chunk ch = chunks[blockIdx.x];
    const Task tk = tasks[ch.task];
    const Split s = splits[ch.task];
    if (threadIdx.x == 0) red = 0;
    __syncthreads();
    int cnt = 0;
    for (int i = ch.begin + threadIdx.x; i < ch.end; i += blockDim.x) {
        int p = ref[i];
        cnt += goes_left(tk, s, i, centroid(plo[p], phi[p])) ? 1 : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(~0u, cnt, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&red, cnt);
    __syncthreads();
    if (threadIdx.x == 0) chunk_left[blockIdx.x] = red;
}

// chunk_lefts_before[c] = lefts of the task's chunks before c.
__global__ void __launch_bounds__(kThreads) k_part_scatter(const Chunk *chunks, const Task *tasks,
                                                           const Split *splits,
                                                           const int *chunk_lefts_before,
                                                           const int *ref, const float4 *plo,
                                                           const float4 *phi, int *ref_out,
                                                           int n, int *err) {
    __shared__ int ws[32];
    const Chunk ch = chunks[blockIdx.x];
    const Task tk = tasks[ch.task];
    const Split s = splits[ch.task];
    int lefts_before = chunk_lefts_before[blockIdx.x];
    for (int base = ch.begin; base < ch.end; base += blockDim.x) {
        int i = base + threadIdx.x;
        bool valid = i < ch.end;
        int p = valid ? ref[i] : 0;
        bool l = valid && goes_left(tk, s, i, centroid(plo[p], phi[p]));
        int tot;
        int rank = block_excl_scan(l ? 1 : 0, ws, &tot);
        if (valid) {
            int lb = lefts_before + rank;  // lefts before position i within the task
            int dst = l ? tk.begin + lb : tk.begin + s.nleft + ((i - tk.begin) - lb);
            if (dst < tk.begin || dst >= tk.begin + tk.count || dst >= n) raise_err(err, kErrBadChild);
            else ref_out[dst] = p;
        }
        lefts_before += tot;
    }
}

__global__ void k_copy_range(const Chunk *chunks, const int *src, int *dst) {
    const Chunk ch = chunks[blockIdx.x];
    for (int i = ch.begin + threadIdx.x; i < ch.end; i += blockDim.x) dst[i] = src[i];
}

// The material class of each BVH-ordered triangle goes into the .w of its
// second record (1 = Disney BRDF, 0 = any other type; the intersection test
// reads only .xyz there), so a closest hit tells the shading queues apart
// without a material lookup.
__global__ void k_tri_class(float4 *tri_rec, int n, const float4 *attr, const kgk_material *mats, int n_mats) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int prim = __float_as_int(tri_rec[3 * i].w);
        const unsigned mid = __float_as_uint(attr[4 * prim + 3].w) & 0x7fffffffu;
        const int cls = mid < (unsigned)n_mats && mats[mid].MATERIAL_TYPE_ID == 1 ? 1 : 0;
        tri_rec[3 * i + 1].w = __int_as_float(cls);
    }
}

__global__ void k_write_nodes(const int *ids, const BinNode *vals, const int *firsts,
                              const int *counts, int m, BinNode *nodes, int *bfirst, int *bcount,
                              int cap, int *err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    int id = ids[i];
    if (id < 0 || id >= cap) { raise_err(err, kErrNodeOverflow); return; }
    nodes[id] = vals[i];
    bfirst[id] = firsts[i];
    bcount[id] = counts[i];
}

// ---------------------------------------------------------------------------
// 3. small tasks: one block builds a whole subtree
// ---------------------------------------------------------------------------
struct SmallEntry {
    int node, b, c, pad;
    float clo[3], chi[3];
};

__global__ void __launch_bounds__(kThreads) k_small_build(const Task *tasks, const int *slot_base,
                                                          const int *slot_end, int ntasks,
                                                          const float4 *__restrict__ plo,
                                                          const float4 *__restrict__ phi, int *ref,
                                                          BinNode *nodes, int *bfirst, int *bcount,
                                                          int cap, int max_leaf, int *err) {
    __shared__ int sref[kSmall];
    __shared__ int stmp[kSmall];
    __shared__ int bins[3 * kBins * kBinInts];
    __shared__ SmallEntry stack[kStack];
    __shared__ int sp;
    __shared__ int ws[32];
    __shared__ WarpSplit best;
    __shared__ SmallEntry cur;
    __shared__ int next_slot;
    __shared__ float red[kThreads / 32][12];

    const int t = blockIdx.x;
    if (t >= ntasks) return;
    const Task tk = tasks[t];
    if (tk.count > kSmall || tk.count < 1) {
        if (threadIdx.x == 0) raise_err(err, kErrSmallTooBig);
        return;
    }
    const int m = tk.count;
    for (int i = threadIdx.x; i < m; i += blockDim.x) sref[i] = ref[tk.begin + i];
    if (threadIdx.x == 0) {
        SmallEntry e;
        e.node = tk.node; e.b = 0; e.c = m;
        for (int a = 0; a < 3; ++a) { e.clo[a] = tk.clo[a]; e.chi[a] = tk.chi[a]; }
        stack[0] = e;
        sp = 1;
        next_slot = slot_base[t];
    }
    __syncthreads();
    const int my_end = slot_end[t];
    __shared__ int stop;
    while (true) {
        __syncthreads();
        const int sp_now = sp;
        __syncthreads();
        if (sp_now == 0) break;
        if (threadIdx.x == 0) cur = stack[--sp];
        __syncthreads();
        const SmallEntry e = cur;
        if (e.node < 0 || e.node >= cap) {  // uniform: every thread reads the same `cur`
            if (threadIdx.x == 0) raise_err(err, kErrNodeOverflow);
            break;
        }
        if (threadIdx.x == 0) {
            bfirst[e.node] = tk.begin + e.b;
            bcount[e.node] = e.c;
        }
        if (e.c <= max_leaf) {
            if (threadIdx.x == 0) {
                nodes[e.node].lo.w = __int_as_float(tk.begin + e.b);
                nodes[e.node].hi.w = __int_as_float(-e.c);
            }
            continue;
        }
        // bin
        float sc[3];
        for (int a = 0; a < 3; ++a) sc[a] = bin_scale(e.clo[a], e.chi[a]);
        init_bins(bins);
        __syncthreads();
        for (int i = threadIdx.x; i < e.c; i += blockDim.x) {
            int p = sref[e.b + i];
            float4 lo = plo[p], hi = phi[p];
            bin_prim(bins, lo, hi, centroid(lo, hi), e.clo, sc, false);
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            WarpSplit w = warp_best_split(bins);
            if (threadIdx.x == 0) best = w;
        }
        __syncthreads();
        const WarpSplit bs = best;
        // stable partition of sref[e.b .. e.b+c)
        int lefts = 0;
        for (int base = 0; base < e.c; base += blockDim.x) {
            int i = base + threadIdx.x;
            bool valid = i < e.c;
            int p = valid ? sref[e.b + i] : 0;
            bool l = false;
            if (valid) {
                if (bs.axis < 0) l = i < e.c / 2;
                else {
                    float3 c = centroid(plo[p], phi[p]);
                    l = bin_of(comp(c, bs.axis), e.clo[bs.axis], sc[bs.axis]) <= bs.bin;
                }
            }
            int tot;
            int rank = block_excl_scan(l ? 1 : 0, ws, &tot);
            if (valid && l) stmp[lefts + rank] = p;
            lefts += tot;
        }
        __syncthreads();
        int nl = lefts;
        int rights = 0;
        for (int base = 0; base < e.c; base += blockDim.x) {
            int i = base + threadIdx.x;
            bool valid = i < e.c;
            int p = valid ? sref[e.b + i] : 0;
            bool r = false;
            if (valid) {
                if (bs.axis < 0) r = !(i < e.c / 2);
                else {
                    float3 c = centroid(plo[p], phi[p]);
                    r = !(bin_of(comp(c, bs.axis), e.clo[bs.axis], sc[bs.axis]) <= bs.bin);
                }
            }
            int tot;
            int rank = block_excl_scan(r ? 1 : 0, ws, &tot);
            if (valid && r) stmp[nl + rights + rank] = p;
            rights += tot;
        }
        __syncthreads();
        if (nl == 0 || nl == e.c) nl = e.c / 2;  // cannot happen with a valid plane; keep the tree finite
        for (int i = threadIdx.x; i < e.c; i += blockDim.x) sref[e.b + i] = stmp[i];
        __syncthreads();
        // exact child boxes and centroid bounds by reduction
        for (int side = 0; side < 2; ++side) {
            int b0 = side == 0 ? 0 : nl, b1 = side == 0 ? nl : e.c;
            float3 lo = f3(INFINITY, INFINITY, INFINITY), hi = f3(-INFINITY, -INFINITY, -INFINITY);
            float3 clo = lo, chi = hi;
            for (int i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
                int p = sref[e.b + i];
                float4 l4 = plo[p], h4 = phi[p];
                lo = fmin3(lo, f3(l4)); hi = fmax3(hi, f3(h4));
                float3 c = centroid(l4, h4);
                clo = fmin3(clo, c); chi = fmax3(chi, c);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                lo = fmin3(lo, f3(__shfl_xor_sync(~0u, lo.x, o), __shfl_xor_sync(~0u, lo.y, o), __shfl_xor_sync(~0u, lo.z, o)));
                hi = fmax3(hi, f3(__shfl_xor_sync(~0u, hi.x, o), __shfl_xor_sync(~0u, hi.y, o), __shfl_xor_sync(~0u, hi.z, o)));
                clo = fmin3(clo, f3(__shfl_xor_sync(~0u, clo.x, o), __shfl_xor_sync(~0u, clo.y, o), __shfl_xor_sync(~0u, clo.z, o)));
                chi = fmax3(chi, f3(__shfl_xor_sync(~0u, chi.x, o), __shfl_xor_sync(~0u, chi.y, o), __shfl_xor_sync(~0u, chi.z, o)));
            }
            const int w = threadIdx.x >> 5;
            if ((threadIdx.x & 31) == 0) {
                red[w][0] = lo.x; red[w][1] = lo.y; red[w][2] = lo.z;
                red[w][3] = hi.x; red[w][4] = hi.y; red[w][5] = hi.z;
                red[w][6] = clo.x; red[w][7] = clo.y; red[w][8] = clo.z;
                red[w][9] = chi.x; red[w][10] = chi.y; red[w][11] = chi.z;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                float r[12];
                for (int k = 0; k < 12; ++k) r[k] = red[0][k];
                for (int ww = 1; ww < kThreads / 32; ++ww)
                    for (int k = 0; k < 12; ++k)
                        r[k] = (k < 3 || (k >= 6 && k < 9)) ? fminf(r[k], red[ww][k]) : fmaxf(r[k], red[ww][k]);
                int id = next_slot + side;
                if (id >= my_end || id >= cap) {
                    raise_err(err, kErrNodeOverflow);
                } else {
                    BinNode nd;
                    nd.lo = make_float4(r[0], r[1], r[2], 0.0f);
                    nd.hi = make_float4(r[3], r[4], r[5], 0.0f);
                    nodes[id] = nd;
                    SmallEntry ce;
                    ce.node = id;
                    ce.b = e.b + b0;
                    ce.c = b1 - b0;
                    for (int a = 0; a < 3; ++a) { ce.clo[a] = r[6 + a]; ce.chi[a] = r[9 + a]; }
                    if (side == 0) cur = ce;
                    else {
                        // push larger first, then smaller (smaller is processed next)
                        SmallEntry le = cur;
                        SmallEntry big = le.c >= ce.c ? le : ce;
                        SmallEntry small = le.c >= ce.c ? ce : le;
                        if (sp + 2 > kStack) {
                            raise_err(err, kErrStackOverflow);
                        } else {
                            stack[sp++] = big;
                            stack[sp++] = small;
                        }
                        nodes[e.node].lo.w = __int_as_float(le.node);
                        nodes[e.node].hi.w = __int_as_float(ce.node);
                    }
                }
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            next_slot += 2;
            stop = *((volatile int *)err);
        }
        __syncthreads();
        if (stop != 0) break;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x) ref[tk.begin + i] = sref[i];
}

// ---------------------------------------------------------------------------
// 4. collapse into 8-wide compressed nodes
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool bn_leaf(const BinNode &n) { return __float_as_int(n.hi.w) < 0; }

// SAH-optimal choice of each wide node's children (Ylitie, Karras and Laine,
// "Efficient incoherent ray traversal on GPUs through compressed wide BVHs",
// HPG 2017, section 3.1).  cost(n, i) is the least SAH cost of the binary
// subtree at n represented as at most i children of a wide node:
//   cost(n, 1) = leaf cost if n may be a leaf (at most max_leaf triangles:
//                c_prim A(n) count), else A(n) c_node + D(n, 8);
//   cost(n, i) = min(cost(n, i - 1), D(n, i)),
//   D(n, j)    = min over 0 < k < j of cost(left, k) + cost(right, j - k).
// The table is filled bottom up, a node by the second of its children to
// finish; dec[n] keeps the argmin k of D(n, 8) (bits 0-2) and, for j = 2..8,
// the k of D(n, j) when it beats cost(n, j - 1), else 0 (bits 3(j-1)..).
constexpr float kCostNode = 1.0f;
constexpr float kCostTri = 0.3f;
constexpr float kCostInf = 3.0e38f;

__global__ void k_dp_parents(const BinNode *nodes, int n_nodes, int *parent, int *err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_nodes) return;
    const BinNode nd = nodes[i];
    if (bn_leaf(nd)) return;  // leaves, and slots no task used (filled with -1)
    const int l = __float_as_int(nd.lo.w), r = __float_as_int(nd.hi.w);
    if (l <= 0 || l >= n_nodes || r <= 0 || r >= n_nodes) { raise_err(err, kErrBadChild); return; }
    parent[l] = i;
    parent[r] = i;
}

__global__ void k_dp_up(const BinNode *nodes, const int *bcount, const int *parent, int n_nodes, int max_leaf,
                        float *cost, unsigned *dec, int *visits, int *err) {
    int node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= n_nodes) return;
    if (!bn_leaf(nodes[node]) || (node != 0 && parent[node] < 0)) return;  // start at the tree's leaves
    {
        const BinNode nd = nodes[node];
        const int cnt = bcount[node];
        const float cl = cnt <= max_leaf ? kCostTri * surface_area(f3(nd.lo), f3(nd.hi)) * (float)cnt : kCostInf;
        for (int j = 0; j < 8; ++j) cost[(size_t)node * 8 + j] = cl;
        dec[node] = 0u;
    }
    for (int guard = 0; guard < 4096; ++guard) {
        const int p = node == 0 ? -1 : parent[node];
        if (p < 0) return;
        __threadfence();
        if (atomicAdd(&visits[p], 1) == 0) return;  // the other child is not done: it finishes p
        __threadfence();
        const BinNode nd = nodes[p];
        const int l = __float_as_int(nd.lo.w), r = __float_as_int(nd.hi.w);
        float cl8[8], cr8[8];
        for (int j = 0; j < 8; ++j) {
            cl8[j] = __ldcg(&cost[(size_t)l * 8 + j]);
            cr8[j] = __ldcg(&cost[(size_t)r * 8 + j]);
        }
        float D[9];
        int K[9];
        D[1] = kCostInf;
        K[1] = 0;
        for (int j = 2; j <= 8; ++j) {
            float best = kCostInf;
            int bk = 1;
            for (int k = 1; k < j; ++k) {
                const float c = cl8[k - 1] + cr8[j - k - 1];
                if (c < best) { best = c; bk = k; }
            }
            D[j] = best;
            K[j] = bk;
        }
        const float area = surface_area(f3(nd.lo), f3(nd.hi));
        const int cnt = bcount[p];
        float c = cnt <= max_leaf ? kCostTri * area * (float)cnt : kCostNode * area + D[8];
        unsigned d = (unsigned)K[8];
        cost[(size_t)p * 8] = c;
        for (int j = 2; j <= 8; ++j) {
            if (D[j] < c) {
                c = D[j];
                d |= (unsigned)K[j] << (3 * (j - 1));
            }
            cost[(size_t)p * 8 + j - 1] = c;
        }
        dec[p] = d;
        node = p;
    }
    raise_err(err, kErrStackOverflow);  // deeper than any tree this build makes
}

__global__ void k_collapse_count(const int *tasks, int ntasks, const BinNode *nodes,
                                 const int *bcount, const unsigned *dec, int *child_list, int *n_inner,
                                 int *n_tris, int cap, int max_leaf, int *err) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks) return;
    int b = tasks[t];
    int C[8];
    int nc = 0;
    if (b < 0 || b >= cap) { raise_err(err, kErrBadChild); return; }
    const BinNode nb = nodes[b];
    if (bcount[b] <= max_leaf || bn_leaf(nb)) {
        C[nc++] = b;
    } else {
        // the 8 slots go to b's two children as the cost table chose, and on
        // down until each share is one slot, a leaf or a node that keeps
        // what it was given
        int sn[16], sj[16];
        int sp = 0;
        const int k8 = (int)(dec[b] & 7u);
        sn[sp] = __float_as_int(nb.lo.w); sj[sp++] = k8;
        sn[sp] = __float_as_int(nb.hi.w); sj[sp++] = 8 - k8;
        while (sp > 0) {
            --sp;
            const int c = sn[sp];
            int j = sj[sp];
            if (c < 0 || c >= cap || j < 1 || nc >= 8) { raise_err(err, kErrBadChild); return; }
            const BinNode nn = nodes[c];
            if (j > 1 && bcount[c] > max_leaf && !bn_leaf(nn)) {
                const unsigned dc = dec[c];
                while (j > 1 && ((dc >> (3 * (j - 1))) & 7u) == 0u) --j;
                if (j > 1) {
                    const int k = (int)((dc >> (3 * (j - 1))) & 7u);
                    if (sp + 2 > 16 || k < 1 || k >= j) { raise_err(err, kErrBadChild); return; }
                    sn[sp] = __float_as_int(nn.lo.w); sj[sp++] = k;
                    sn[sp] = __float_as_int(nn.hi.w); sj[sp++] = j - k;
                    continue;
                }
            }
            C[nc++] = c;
        }
    }
    int ni = 0, nt = 0;
    for (int i = 0; i < 8; ++i) {
        int c = i < nc ? C[i] : -1;
        child_list[t * 8 + i] = c;
        if (c >= 0) {
            if (c >= cap) { raise_err(err, kErrBadChild); return; }
            int k = bcount[c];
            if (k <= max_leaf) nt += k;
            else ni += 1;
        }
    }
    n_inner[t] = ni;
    n_tris[t] = nt;
}

// Per-axis quantisation exponent: the smallest power of two s with
// extent / s <= 255, returned as the biased exponent byte.
__device__ __forceinline__ int quant_exponent(float extent) {
    if (!(extent > 0.0f)) return 27;  // 2^-100: a flat axis
    float r = extent / 255.0f;
    int e;
    frexpf(r, &e);  // r = m * 2^e, m in [0.5, 1)
    int k = e;      // 2^e >= r
    if (ldexpf(1.0f, k - 1) >= r) k -= 1;
    while (extent / ldexpf(1.0f, k) > 255.0f) ++k;
    if (k < -100) k = -100;
    return k + 127;
}

__global__ void k_collapse_emit(const int *tasks, int ntasks, const int *child_list,
                                const int *inner_scan, const int *tri_scan, int level_start,
                                int next_start, int tri_start, const BinNode *nodes, int cap,
                                const int *bfirst, const int *bcount, const int *ref,
                                const float4 *verts, WideNode *wide, int wide_cap, float4 *tri_rec,
                                int n_tris, int *next_tasks, int next_cap, int max_leaf, int *err) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks) return;
    int C[8];
    float3 clo[8], chi[8];
    int nc = 0;
    float3 plo = f3(INFINITY, INFINITY, INFINITY), phi = f3(-INFINITY, -INFINITY, -INFINITY);
    for (int i = 0; i < 8; ++i) {
        int c = child_list[t * 8 + i];
        if (c < 0) continue;
        if (c >= cap) { raise_err(err, kErrBadChild); return; }
        C[nc] = c;
        clo[nc] = f3(nodes[c].lo);
        chi[nc] = f3(nodes[c].hi);
        plo = fmin3(plo, clo[nc]);
        phi = fmax3(phi, chi[nc]);
        ++nc;
    }
    // slot assignment: child i -> slot s maximising dot(centre_i - centre, D(s)),
    // D(s) = (s&4 ? +1 : -1, s&2 ? +1 : -1, s&1 ? +1 : -1); greedy over pairs.
    float3 pc = 0.5f * (plo + phi);
    int slot_of[8];
    int child_in_slot[8];
    for (int i = 0; i < 8; ++i) { slot_of[i] = -1; child_in_slot[i] = -1; }
    for (int round = 0; round < nc; ++round) {
        float bestv = -INFINITY;
        int bi = -1, bsl = -1;
        for (int i = 0; i < nc; ++i) {
            if (slot_of[i] >= 0) continue;
            float3 d = 0.5f * (clo[i] + chi[i]) - pc;
            for (int s = 0; s < 8; ++s) {
                if (child_in_slot[s] >= 0) continue;
                float v = ((s & 4) ? d.x : -d.x) + ((s & 2) ? d.y : -d.y) + ((s & 1) ? d.z : -d.z);
                if (v > bestv) { bestv = v; bi = i; bsl = s; }
            }
        }
        slot_of[bi] = bsl;
        child_in_slot[bsl] = bi;
    }
    // quantisation frame
    float3 ext = (phi - plo) * (1.0f + 1.0f / 1048576.0f);
    int ex = quant_exponent(ext.x), ey = quant_exponent(ext.y), ez = quant_exponent(ext.z);
    float sx = ldexpf(1.0f, ex - 127), sy = ldexpf(1.0f, ey - 127), sz = ldexpf(1.0f, ez - 127);
    unsigned meta[8], qlx[8], qly[8], qlz[8], qhx[8], qhy[8], qhz[8];
    unsigned imask = 0;
    const int child_base = next_start + inner_scan[t];
    const int tri_base = tri_start + tri_scan[t];
    int inner_k = 0, tri_off = 0;
    for (int s = 0; s < 8; ++s) {
        int i = child_in_slot[s];
        meta[s] = 0;
        qlx[s] = qly[s] = qlz[s] = 0;
        qhx[s] = qhy[s] = qhz[s] = 0;
        if (i < 0) continue;
        int c = C[i];
        int k = bcount[c];
        // conservative quantisation
        float q;
        q = floorf((clo[i].x - plo.x) / sx); while (q > 0.0f && plo.x + q * sx > clo[i].x) q -= 1.0f; qlx[s] = (unsigned)fminf(fmaxf(q, 0.0f), 255.0f);
        q = floorf((clo[i].y - plo.y) / sy); while (q > 0.0f && plo.y + q * sy > clo[i].y) q -= 1.0f; qly[s] = (unsigned)fminf(fmaxf(q, 0.0f), 255.0f);
        q = floorf((clo[i].z - plo.z) / sz); while (q > 0.0f && plo.z + q * sz > clo[i].z) q -= 1.0f; qlz[s] = (unsigned)fminf(fmaxf(q, 0.0f), 255.0f);
        q = ceilf((chi[i].x - plo.x) / sx); while (q < 255.0f && plo.x + q * sx < chi[i].x) q += 1.0f; qhx[s] = (unsigned)fminf(fmaxf(q, 0.0f), 255.0f);
        q = ceilf((chi[i].y - plo.y) / sy); while (q < 255.0f && plo.y + q * sy < chi[i].y) q += 1.0f; qhy[s] = (unsigned)fminf(fmaxf(q, 0.0f), 255.0f);
        q = ceilf((chi[i].z - plo.z) / sz); while (q < 255.0f && plo.z + q * sz < chi[i].z) q += 1.0f; qhz[s] = (unsigned)fminf(fmaxf(q, 0.0f), 255.0f);
        if (k > max_leaf) {
            int wid = child_base + inner_k;
            int pos = inner_scan[t] + inner_k;
            if (pos >= next_cap || wid >= wide_cap) { raise_err(err, kErrWideOverflow); return; }
            next_tasks[pos] = c;
            meta[s] = 0x20u | (unsigned)(24 + s);
            imask |= 1u << s;
            ++inner_k;
        } else {
            if (tri_off + k > 24 || tri_base + tri_off + k > n_tris) { raise_err(err, kErrTriOverflow); return; }
            unsigned unary = k == 1 ? 1u : (k == 2 ? 3u : 7u);
            meta[s] = (unary << 5) | (unsigned)tri_off;
            int f = bfirst[c];
            if (f < 0 || f + k > n_tris) { raise_err(err, kErrTriOverflow); return; }
            for (int j = 0; j < k; ++j) {
                int prim = ref[f + j];
                if (prim < 0 || prim >= n_tris) { raise_err(err, kErrTriOverflow); return; }
                int dst = tri_base + tri_off + j;
                float4 a = verts[3 * prim], b = verts[3 * prim + 1], cc = verts[3 * prim + 2];
                tri_rec[3 * dst] = make_float4(a.x, a.y, a.z, __int_as_float(prim));
                tri_rec[3 * dst + 1] = make_float4(b.x, b.y, b.z, 0.0f);
                tri_rec[3 * dst + 2] = make_float4(cc.x, cc.y, cc.z, 0.0f);
            }
            tri_off += k;
        }
    }
    int me = level_start + t;
    if (me >= wide_cap) { raise_err(err, kErrWideOverflow); return; }
    auto pack4 = [](const unsigned *v, int o) {
        return v[o] | (v[o + 1] << 8) | (v[o + 2] << 16) | (v[o + 3] << 24);
    };
    WideNode w;
    w.n0 = make_float4(plo.x, plo.y, plo.z,
                       __uint_as_float((unsigned)ex | ((unsigned)ey << 8) | ((unsigned)ez << 16) | (imask << 24)));
    w.n1 = make_float4(__int_as_float(child_base), __int_as_float(tri_base),
                       __uint_as_float(pack4(meta, 0)), __uint_as_float(pack4(meta, 4)));
    w.n2 = make_float4(__uint_as_float(pack4(qlx, 0)), __uint_as_float(pack4(qlx, 4)),
                       __uint_as_float(pack4(qhx, 0)), __uint_as_float(pack4(qhx, 4)));
    w.n3 = make_float4(__uint_as_float(pack4(qly, 0)), __uint_as_float(pack4(qly, 4)),
                       __uint_as_float(pack4(qhy, 0)), __uint_as_float(pack4(qhy, 4)));
    w.n4 = make_float4(__uint_as_float(pack4(qlz, 0)), __uint_as_float(pack4(qlz, 4)),
                       __uint_as_float(pack4(qhz, 0)), __uint_as_float(pack4(qhz, 4)));
    wide[me] = w;
}

// ---------------------------------------------------------------------------
// device-wide exclusive scan of ints (3 phases)
// ---------------------------------------------------------------------------
constexpr int kScanBlock = 1024;  // elements per block (4 per thread)

__global__ void k_scan_local(const int *in, int *out, int n, int *block_sums) {
    __shared__ int ws[32];
    const int base = blockIdx.x * kScanBlock + threadIdx.x * 4;
    int v[4], s = 0;
    for (int k = 0; k < 4; ++k) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    int tot;
    int ex = block_excl_scan(s, ws, &tot);
    for (int k = 0; k < 4; ++k) {
        if (base + k < n) out[base + k] = ex;
        ex += v[k];
    }
    if (threadIdx.x == 0 && block_sums) block_sums[blockIdx.x] = tot;
}

__global__ void k_scan_add(int *out, int n, const int *block_offsets) {
    const int base = blockIdx.x * kScanBlock + threadIdx.x * 4;
    const int off = block_offsets[blockIdx.x];
    for (int k = 0; k < 4; ++k)
        if (base + k < n) out[base + k] += off;
}

struct ScanTmp {
    std::vector<int *> levels;
};

// Exclusive scan of n ints; *total (host) gets the sum.  tmp must hold
// scan_tmp_ints(n) ints.
size_t scan_tmp_ints(int n) {
    size_t s = 0;
    while (n > kScanBlock) {
        n = (n + kScanBlock - 1) / kScanBlock;
        s += 2 * (size_t)n + 4;
    }
    return s + 8;
}

kgk_status scan_exclusive(const int *in, int *out, int n, int *tmp, int *total_dev,
                          cudaStream_t st) {
    if (n <= 0) return KGK_OK;
    int nb = (n + kScanBlock - 1) / kScanBlock;
    if (nb == 1) {
        k_scan_local<<<1, 256, 0, st>>>(in, out, n, total_dev);
        KGK_CUDA(cudaGetLastError());
        return KGK_OK;
    }
    int *sums = tmp;
    int *offs = tmp + nb;
    k_scan_local<<<nb, 256, 0, st>>>(in, out, n, sums);
    KGK_CUDA(cudaGetLastError());
    KGK_TRY(scan_exclusive(sums, offs, nb, tmp + 2 * nb + 4, total_dev, st));
    k_scan_add<<<nb, 256, 0, st>>>(out, n, offs);
    KGK_CUDA(cudaGetLastError());
    return KGK_OK;
}

float host_f(int i) { float f; memcpy(&f, &i, 4); return f; }
float host_o2f(int i) { return host_f(i >= 0 ? i : i ^ 0x7fffffff); }

struct DevBuf {
    std::vector<void *> ptrs;
    ~DevBuf() {
        for (void *p : ptrs) dfree(p);
    }
    template <class T> kgk_status get(T **p, size_t count, const char *what) {
        KGK_TRY(dalloc(p, count > 0 ? count : 1, what));
        ptrs.push_back(*p);
        return KGK_OK;
    }
};

}  // namespace

// ---------------------------------------------------------------------------
kgk_status bvh_build(DevScene &s, cudaStream_t st, BvhBuildStats *out) {
    const int n = s.n_tris;
    if (n <= 0) return fail(KGK_ERR_INVALID_ARGUMENT, "bvh_build: scene has no triangles");
    const int max_leaf = n > kLargeSceneTris ? kLeafLarge : kMaxLeaf;
    dfree(s.nodes);
    s.nodes = nullptr;
    dfree(s.tri_rec);
    s.tri_rec = nullptr;
    s.n_nodes = 0;

    cudaEvent_t e0, e1;
    KGK_CUDA(cudaEventCreate(&e0));
    KGK_CUDA(cudaEventCreate(&e1));
    KGK_CUDA(cudaEventRecord(e0, st));

    DevBuf buf;
    float4 *plo, *phi;
    int *ref, *ref_tmp, *gbounds, *err, *bfirst, *bcount;
    BinNode *nodes;
    const int cap = 2 * n + 1;
    KGK_TRY(buf.get(&plo, n, "bvh prim boxes"));
    KGK_TRY(buf.get(&phi, n, "bvh prim boxes"));
    KGK_TRY(buf.get(&ref, n, "bvh refs"));
    KGK_TRY(buf.get(&ref_tmp, n, "bvh refs"));
    KGK_TRY(buf.get(&gbounds, 16, "bvh bounds"));
    KGK_TRY(buf.get(&err, 4, "bvh error flag"));
    KGK_TRY(buf.get(&nodes, cap, "bvh binary nodes"));
    KGK_TRY(buf.get(&bfirst, cap, "bvh binary nodes"));
    KGK_TRY(buf.get(&bcount, cap, "bvh binary nodes"));
    // slots the small builder reserves but does not use read as leaves
    // (hi.w = -1) that no node points to
    KGK_CUDA(cudaMemsetAsync(nodes, 0xFF, (size_t)cap * sizeof(BinNode), st));
    KGK_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));

    k_init_bounds<<<1, 32, 0, st>>>(gbounds);
    k_prim_bounds<<<(n + 255) / 256, 256, 0, st>>>(s.verts, n, plo, phi, ref, gbounds);
    KGK_CUDA(cudaGetLastError());
    int hb[12];
    KGK_CUDA(cudaMemcpyAsync(hb, gbounds, sizeof hb, cudaMemcpyDeviceToHost, st));
    KGK_CUDA(cudaStreamSynchronize(st));

    // root
    Task root{};
    root.node = 0;
    root.begin = 0;
    root.count = n;
    for (int a = 0; a < 3; ++a) {
        root.clo[a] = host_o2f(hb[6 + a]);
        root.chi[a] = host_o2f(hb[9 + a]);
    }
    std::vector<int> h_ids;
    std::vector<BinNode> h_vals;
    std::vector<int> h_first, h_count;
    auto add_node = [&](int id, const float *lo, const float *hi, int first, int count) {
        BinNode nd;
        nd.lo = make_float4(lo[0], lo[1], lo[2], 0.0f);
        nd.hi = make_float4(hi[0], hi[1], hi[2], 0.0f);
        h_ids.push_back(id);
        h_vals.push_back(nd);
        h_first.push_back(first);
        h_count.push_back(count);
        return (int)h_ids.size() - 1;
    };
    float rlo[3] = {host_o2f(hb[0]), host_o2f(hb[1]), host_o2f(hb[2])};
    float rhi[3] = {host_o2f(hb[3]), host_o2f(hb[4]), host_o2f(hb[5])};
    add_node(0, rlo, rhi, 0, n);
    int node_counter = 1;

    std::vector<Task> large, small;
    if (n > kSmall) large.push_back(root);
    else small.push_back(root);

    Task *d_tasks = nullptr;
    Split *d_splits = nullptr;
    Chunk *d_chunks = nullptr;
    int *d_gbins = nullptr, *d_chunk_left = nullptr, *d_before = nullptr;
    const int max_large = n / kSmall + 2;
    const int max_chunks = n / kChunk + 2 * max_large + 2;
    KGK_TRY(buf.get(&d_tasks, std::max(max_large, 1), "bvh tasks"));
    KGK_TRY(buf.get(&d_splits, std::max(max_large, 1), "bvh splits"));
    KGK_TRY(buf.get(&d_chunks, max_chunks, "bvh chunks"));
    KGK_TRY(buf.get(&d_gbins, (size_t)std::max(max_large, 1) * 3 * kBins * kBinInts, "bvh bins"));
    KGK_TRY(buf.get(&d_chunk_left, max_chunks, "bvh chunk counts"));
    KGK_TRY(buf.get(&d_before, max_chunks, "bvh chunk counts"));

    int levels = 0;
    while (!large.empty()) {
        ++levels;
        const int nL = (int)large.size();
        if (nL > max_large) return fail(KGK_ERR_DEVICE_CHECK, "bvh_build: large-task list overflow");
        std::vector<Chunk> chunks;
        for (int t = 0; t < nL; ++t)
            for (int b = large[t].begin; b < large[t].begin + large[t].count; b += kChunk)
                chunks.push_back({t, b, std::min(b + kChunk, large[t].begin + large[t].count), 0});
        const int nc = (int)chunks.size();
        if (nc > max_chunks) return fail(KGK_ERR_DEVICE_CHECK, "bvh_build: chunk list overflow");
        KGK_CUDA(cudaMemcpyAsync(d_tasks, large.data(), sizeof(Task) * nL, cudaMemcpyHostToDevice, st));
        KGK_CUDA(cudaMemcpyAsync(d_chunks, chunks.data(), sizeof(Chunk) * nc, cudaMemcpyHostToDevice, st));
        const int nbins = nL * 3 * kBins * kBinInts;
        k_init_global_bins<<<(nbins + 255) / 256, 256, 0, st>>>(d_gbins, nL);
        k_bin_large<<<nc, kThreads, 0, st>>>(d_chunks, d_tasks, ref, plo, phi, d_gbins);
        k_split_large<<<nL, 32, 0, st>>>(d_tasks, nL, d_gbins, d_splits);
        k_part_count<<<nc, kThreads, 0, st>>>(d_chunks, d_tasks, d_splits, ref, plo, phi, d_chunk_left);
        KGK_CUDA(cudaGetLastError());
        std::vector<int> cl(nc);
        std::vector<Split> sp(nL);
        KGK_CUDA(cudaMemcpyAsync(cl.data(), d_chunk_left, sizeof(int) * nc, cudaMemcpyDeviceToHost, st));
        KGK_CUDA(cudaMemcpyAsync(sp.data(), d_splits, sizeof(Split) * nL, cudaMemcpyDeviceToHost, st));
        KGK_CUDA(cudaStreamSynchronize(st));
        std::vector<int> before(nc);
        std::vector<int> task_left(nL, 0);
        for (int c = 0; c < nc; ++c) {
            before[c] = task_left[chunks[c].task];
            task_left[chunks[c].task] += cl[c];
        }
        for (int t = 0; t < nL; ++t) {
            if (sp[t].axis >= 0 && task_left[t] != sp[t].nleft)
                return fail(KGK_ERR_DEVICE_CHECK, "bvh_build: partition count disagrees with the bins");
            if (sp[t].axis < 0) sp[t].nleft = large[t].count / 2;
        }
        KGK_CUDA(cudaMemcpyAsync(d_before, before.data(), sizeof(int) * nc, cudaMemcpyHostToDevice, st));
        k_part_scatter<<<nc, kThreads, 0, st>>>(d_chunks, d_tasks, d_splits, d_before, ref, plo, phi,
                                                 ref_tmp, n, err);
        k_copy_range<<<nc, kThreads, 0, st>>>(d_chunks, ref_tmp, ref);
        KGK_CUDA(cudaGetLastError());
        std::vector<Task> next;
        for (int t = 0; t < nL; ++t) {
            const Task &tk = large[t];
            const Split &s2 = sp[t];
            const int l = node_counter, r = node_counter + 1;
            node_counter += 2;
            // parent's child links
            int pi = -1;
            for (int k = (int)h_ids.size() - 1; k >= 0; --k)
                if (h_ids[k] == tk.node) { pi = k; break; }
            if (pi < 0) return fail(KGK_ERR_DEVICE_CHECK, "bvh_build: lost a parent node");
            h_vals[pi].lo.w = host_f(l);
            h_vals[pi].hi.w = host_f(r);
            for (int side = 0; side < 2; ++side) {
                Task c{};
                c.node = side == 0 ? l : r;
                c.begin = side == 0 ? tk.begin : tk.begin + s2.nleft;
                c.count = side == 0 ? s2.nleft : tk.count - s2.nleft;
                for (int a = 0; a < 3; ++a) { c.clo[a] = s2.clo[side][a]; c.chi[a] = s2.chi[side][a]; }
                add_node(c.node, s2.lo[side], s2.hi[side], c.begin, c.count);
                if (c.count > kSmall) next.push_back(c);
                else small.push_back(c);
            }
        }
        large.swap(next);
    }

    // upload the large-level nodes (before the small kernel links into them)
    {
        const int m = (int)h_ids.size();
        int *d_ids, *d_first, *d_count;
        BinNode *d_vals;
        KGK_TRY(buf.get(&d_ids, m, "bvh node staging"));
        KGK_TRY(buf.get(&d_first, m, "bvh node staging"));
        KGK_TRY(buf.get(&d_count, m, "bvh node staging"));
        KGK_TRY(buf.get(&d_vals, m, "bvh node staging"));
        KGK_CUDA(cudaMemcpyAsync(d_ids, h_ids.data(), sizeof(int) * m, cudaMemcpyHostToDevice, st));
        KGK_CUDA(cudaMemcpyAsync(d_first, h_first.data(), sizeof(int) * m, cudaMemcpyHostToDevice, st));
        KGK_CUDA(cudaMemcpyAsync(d_count, h_count.data(), sizeof(int) * m, cudaMemcpyHostToDevice, st));
        KGK_CUDA(cudaMemcpyAsync(d_vals, h_vals.data(), sizeof(BinNode) * m, cudaMemcpyHostToDevice, st));
        k_write_nodes<<<(m + 255) / 256, 256, 0, st>>>(d_ids, d_vals, d_first, d_count, m, nodes,
                                                       bfirst, bcount, cap, err);
        KGK_CUDA(cudaGetLastError());
        KGK_CUDA(cudaStreamSynchronize(st));
    }

    // small subtrees: each task of m primitives owns 2m-2 node slots
    if (!small.empty()) {
        const int ns = (int)small.size();
        std::vector<int> sb(ns), se(ns);
        long long next = node_counter;
        for (int t = 0; t < ns; ++t) {
            sb[t] = (int)next;
            next += 2LL * small[t].count - 2;
            se[t] = (int)next;
        }
        if (next > cap) return fail(KGK_ERR_DEVICE_CHECK, "bvh_build: node budget exceeded");
        node_counter = (int)next;
        Task *d_small;
        int *d_sb, *d_se;
        KGK_TRY(buf.get(&d_small, ns, "bvh small tasks"));
        KGK_TRY(buf.get(&d_sb, ns, "bvh small tasks"));
        KGK_TRY(buf.get(&d_se, ns, "bvh small tasks"));
        KGK_CUDA(cudaMemcpyAsync(d_small, small.data(), sizeof(Task) * ns, cudaMemcpyHostToDevice, st));
        KGK_CUDA(cudaMemcpyAsync(d_sb, sb.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, st));
        KGK_CUDA(cudaMemcpyAsync(d_se, se.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, st));
        k_small_build<<<ns, kThreads, 0, st>>>(d_small, d_sb, d_se, ns, plo, phi, ref, nodes, bfirst,
                                               bcount, cap, max_leaf, err);
        KGK_CUDA(cudaGetLastError());
    }
    int herr = 0;
    KGK_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    KGK_CUDA(cudaStreamSynchronize(st));
    if (herr != 0)
        return fail(KGK_ERR_DEVICE_CHECK, "bvh_build: binary build check failed (code " + std::to_string(herr) + ")");

    // the collapse's cost table, bottom up over the binary tree
    const int n_bin = node_counter;
    int *parent, *visits;
    float *dp_cost;
    unsigned *dec;
    KGK_TRY(buf.get(&parent, n_bin, "bvh collapse table"));
    KGK_TRY(buf.get(&visits, n_bin, "bvh collapse table"));
    KGK_TRY(buf.get(&dp_cost, 8 * (size_t)n_bin, "bvh collapse table"));
    KGK_TRY(buf.get(&dec, n_bin, "bvh collapse table"));
    KGK_CUDA(cudaMemsetAsync(parent, 0xFF, (size_t)n_bin * sizeof(int), st));
    KGK_CUDA(cudaMemsetAsync(visits, 0, (size_t)n_bin * sizeof(int), st));
    KGK_CUDA(cudaMemsetAsync(dec, 0, (size_t)n_bin * sizeof(unsigned), st));
    k_dp_parents<<<(n_bin + 255) / 256, 256, 0, st>>>(nodes, n_bin, parent, err);
    k_dp_up<<<(n_bin + 255) / 256, 256, 0, st>>>(nodes, bcount, parent, n_bin, max_leaf, dp_cost, dec, visits, err);
    KGK_CUDA(cudaGetLastError());

    // collapse
    WideNode *wide;
    float4 *tri_rec;
    const int wide_cap = n + 1;
    KGK_TRY(dalloc(&wide, wide_cap, "wide BVH nodes"));
    s.nodes = wide;
    KGK_TRY(dalloc(&tri_rec, 3 * (size_t)n, "BVH triangle records"));
    s.tri_rec = tri_rec;
    int *tasks_a, *tasks_b, *child_list, *n_inner, *n_tri, *inner_scan, *tri_scan, *scan_tmp, *tot;
    KGK_TRY(buf.get(&tasks_a, wide_cap, "collapse tasks"));
    KGK_TRY(buf.get(&tasks_b, wide_cap, "collapse tasks"));
    KGK_TRY(buf.get(&child_list, 8 * (size_t)wide_cap, "collapse children"));
    KGK_TRY(buf.get(&n_inner, wide_cap, "collapse counts"));
    KGK_TRY(buf.get(&n_tri, wide_cap, "collapse counts"));
    KGK_TRY(buf.get(&inner_scan, wide_cap, "collapse scans"));
    KGK_TRY(buf.get(&tri_scan, wide_cap, "collapse scans"));
    KGK_TRY(buf.get(&scan_tmp, scan_tmp_ints(wide_cap), "scan scratch"));
    KGK_TRY(buf.get(&tot, 4, "scan totals"));
    int zero = 0;
    KGK_CUDA(cudaMemcpyAsync(tasks_a, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
    int ntasks = 1, level_start = 0, tri_start = 0, wlevels = 0;
    while (ntasks > 0) {
        ++wlevels;
        const int g = (ntasks + 127) / 128;
        k_collapse_count<<<g, 128, 0, st>>>(tasks_a, ntasks, nodes, bcount, dec, child_list, n_inner, n_tri,
                                            cap, max_leaf, err);
        KGK_CUDA(cudaGetLastError());
        KGK_TRY(scan_exclusive(n_inner, inner_scan, ntasks, scan_tmp, tot, st));
        KGK_TRY(scan_exclusive(n_tri, tri_scan, ntasks, scan_tmp, tot + 1, st));
        // totals: last exclusive value + last count
        int h[5];
        KGK_CUDA(cudaMemcpyAsync(&h[4], err, sizeof(int), cudaMemcpyDeviceToHost, st));
        KGK_CUDA(cudaMemcpyAsync(&h[0], inner_scan + ntasks - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        KGK_CUDA(cudaMemcpyAsync(&h[1], n_inner + ntasks - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        KGK_CUDA(cudaMemcpyAsync(&h[2], tri_scan + ntasks - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        KGK_CUDA(cudaMemcpyAsync(&h[3], n_tri + ntasks - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        KGK_CUDA(cudaStreamSynchronize(st));
        if (h[4] != 0)
            return fail(KGK_ERR_DEVICE_CHECK, "bvh_build: collapse check failed (code " + std::to_string(h[4]) + ")");
        const int next_n = h[0] + h[1];
        const int level_tris = h[2] + h[3];
        const int next_start = level_start + ntasks;
        if (next_start + next_n > wide_cap || tri_start + level_tris > n)
            return fail(KGK_ERR_DEVICE_CHECK, "bvh_build: collapse exceeded its budget");
        k_collapse_emit<<<g, 128, 0, st>>>(tasks_a, ntasks, child_list, inner_scan, tri_scan,
                                           level_start, next_start, tri_start, nodes, cap, bfirst, bcount,
                                           ref, s.verts, wide, wide_cap, tri_rec, n, tasks_b,
                                           wide_cap, max_leaf, err);
        KGK_CUDA(cudaGetLastError());
        level_start = next_start;
        tri_start += level_tris;
        ntasks = next_n;
        std::swap(tasks_a, tasks_b);
    }
    if (tri_start == n) {
        k_tri_class<<<std::min((n + 255) / 256, 4096), 256, 0, st>>>(tri_rec, n, s.attr, s.mats, s.n_mats);
        KGK_CUDA(cudaGetLastError());
    }
    KGK_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    KGK_CUDA(cudaEventRecord(e1, st));
    KGK_CUDA(cudaStreamSynchronize(st));
    if (herr != 0)
        return fail(KGK_ERR_DEVICE_CHECK, "bvh_build: collapse check failed (code " + std::to_string(herr) + ")");
    if (tri_start != n)
        return fail(KGK_ERR_DEVICE_CHECK, "bvh_build: collapse placed " + std::to_string(tri_start) +
                                              " of " + std::to_string(n) + " triangles");
    s.n_nodes = level_start;
    s.root = 0;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (out) {
        out->n_binary = (uint64_t)node_counter;
        out->n_wide = (uint64_t)s.n_nodes;
        out->max_depth = (uint32_t)wlevels;
        out->max_leaf = max_leaf;
        out->ms = ms;
        out->sah = 0;
    }
    return KGK_OK;
}

// ---------------------------------------------------------------------------
// Host-side structural validation of the wide BVH.
// ---------------------------------------------------------------------------
kgk_status bvh_validate(const DevScene &s, cudaStream_t st) {
    if (!s.nodes || !s.tri_rec) return fail(KGK_ERR_NOT_BUILT, "bvh_validate: no BVH");
    const int n = s.n_tris;
    std::vector<WideNode> nodes(s.n_nodes);
    std::vector<float4> tri(3 * (size_t)n);
    KGK_CUDA(cudaMemcpyAsync(nodes.data(), s.nodes, sizeof(WideNode) * nodes.size(), cudaMemcpyDeviceToHost, st));
    KGK_CUDA(cudaMemcpyAsync(tri.data(), s.tri_rec, sizeof(float4) * tri.size(), cudaMemcpyDeviceToHost, st));
    KGK_CUDA(cudaStreamSynchronize(st));
    std::vector<int> seen(n, 0);
    std::vector<int> visited(nodes.size(), 0);
    struct Item { int node; float lo[3], hi[3]; };
    std::vector<Item> stack;
    Item root{0, {-INFINITY, -INFINITY, -INFINITY}, {INFINITY, INFINITY, INFINITY}};
    stack.push_back(root);
    auto u = [](float f) { unsigned x; memcpy(&x, &f, 4); return x; };
    auto byte = [](unsigned w, int k) { return (w >> (8 * k)) & 0xffu; };
    while (!stack.empty()) {
        Item it = stack.back();
        stack.pop_back();
        if (it.node < 0 || it.node >= (int)nodes.size())
            return fail(KGK_ERR_DEVICE_CHECK, "bvh_validate: child index out of range");
        if (visited[it.node]++) return fail(KGK_ERR_DEVICE_CHECK, "bvh_validate: node reached twice");
        const WideNode &w = nodes[it.node];
        float p[3] = {w.n0.x, w.n0.y, w.n0.z};
        unsigned e = u(w.n0.w);
        float sc[3];
        for (int a = 0; a < 3; ++a) sc[a] = ldexpf(1.0f, (int)byte(e, a) - 127);
        unsigned imask = byte(e, 3);
        int child_base = (int)u(w.n1.x), tri_base = (int)u(w.n1.y);
        unsigned meta_w[2] = {u(w.n1.z), u(w.n1.w)};
        unsigned ql[3][2] = {{u(w.n2.x), u(w.n2.y)}, {u(w.n3.x), u(w.n3.y)}, {u(w.n4.x), u(w.n4.y)}};
        unsigned qh[3][2] = {{u(w.n2.z), u(w.n2.w)}, {u(w.n3.z), u(w.n3.w)}, {u(w.n4.z), u(w.n4.w)}};
        int inner_k = 0;
        for (int sl = 0; sl < 8; ++sl) {
            unsigned meta = byte(meta_w[sl / 4], sl % 4);
            if (meta == 0) continue;
            float lo[3], hi[3];
            for (int a = 0; a < 3; ++a) {
                lo[a] = p[a] + (float)byte(ql[a][sl / 4], sl % 4) * sc[a];
                hi[a] = p[a] + (float)byte(qh[a][sl / 4], sl % 4) * sc[a];
                if (lo[a] > hi[a]) return fail(KGK_ERR_DEVICE_CHECK, "bvh_validate: inverted child box");
            }
            if ((meta & 0x1f) >= 24) {
                if (!(imask & (1u << sl)) || (meta & 0x1f) != 24u + sl)
                    return fail(KGK_ERR_DEVICE_CHECK, "bvh_validate: inner meta inconsistent");
                Item c;
                c.node = child_base + inner_k++;
                for (int a = 0; a < 3; ++a) { c.lo[a] = lo[a]; c.hi[a] = hi[a]; }
                stack.push_back(c);
            } else {
                unsigned unary = meta >> 5;
                int k = unary == 1 ? 1 : (unary == 3 ? 2 : (unary == 7 ? 3 : 0));
                if (k == 0) return fail(KGK_ERR_DEVICE_CHECK, "bvh_validate: bad leaf meta");
                for (int j = 0; j < k; ++j) {
                    int ti = tri_base + (int)(meta & 0x1f) + j;
                    if (ti < 0 || ti >= n) return fail(KGK_ERR_DEVICE_CHECK, "bvh_validate: triangle index out of range");
                    int id;
                    memcpy(&id, &tri[3 * (size_t)ti].w, 4);
                    if (id < 0 || id >= n || seen[id]++) return fail(KGK_ERR_DEVICE_CHECK, "bvh_validate: triangle referenced twice");
                    for (int v = 0; v < 3; ++v) {
                        const float4 &q = tri[3 * (size_t)ti + v];
                        float c3[3] = {q.x, q.y, q.z};
                        for (int a = 0; a < 3; ++a) {
                            float tol = 1e-6f * (fabsf(c3[a]) + 1.0f);
                            if (c3[a] < lo[a] - tol || c3[a] > hi[a] + tol)
                                return fail(KGK_ERR_DEVICE_CHECK, "bvh_validate: triangle outside its leaf box");
                        }
                    }
                }
            }
        }
        if (__builtin_popcount(imask) != inner_k) return fail(KGK_ERR_DEVICE_CHECK, "bvh_validate: imask count mismatch");
    }
    for (int i = 0; i < n; ++i)
        if (seen[i] != 1) return fail(KGK_ERR_DEVICE_CHECK, "bvh_validate: triangle " + std::to_string(i) + " not referenced");
    for (size_t i = 0; i < nodes.size(); ++i)
        if (!visited[i]) return fail(KGK_ERR_DEVICE_CHECK, "bvh_validate: unreachable node");
    return KGK_OK;
}

}  // namespace kgk
