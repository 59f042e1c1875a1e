// trace.cu - batch closest-hit and occlusion queries (the parity entry
// points kgk_trace_closest / kgk_trace_any): persistent kernels, one ray per
// lane at a time, lanes refilled from a shared counter.
#include <algorithm>

#include "kgk_internal.h"
#include "traverse.cuh"

namespace kgk {
namespace {

// kgk_ray is 40 B (dir, org, double): rays are read as five float2.
__device__ __forceinline__ void load_ray(const kgk_ray *rays, int i, float3 &o, float3 &d) {
    const float2 *p = reinterpret_cast<const float2 *>(reinterpret_cast<const char *>(rays) + 40 * (size_t)i);
    const float2 a = p[0], b = p[1], c = p[2], e = p[3];
    d = f3(a.x, a.y, b.x);
    o = f3(c.x, c.y, e.x);
}

__device__ __forceinline__ void flush_counters(TraceCounters *ctr, unsigned nodes, unsigned tris,
                                               unsigned overflow, unsigned rays) {
    unsigned long long n = nodes, t = tris, o = overflow, r = rays;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        n += __shfl_xor_sync(~0u, n, s);
        t += __shfl_xor_sync(~0u, t, s);
        o += __shfl_xor_sync(~0u, o, s);
        r += __shfl_xor_sync(~0u, r, s);
    }
    if ((threadIdx.x & 31) == 0) {
        if (r) atomicAdd(&ctr->rays, r);
        if (o) atomicAdd(&ctr->overflows, o);
        if (n) atomicAdd(&ctr->nodes, n);
        if (t) atomicAdd(&ctr->tris, t);
    }
}

// Lanes take new rays (one atomic per warp) whenever kRefill or more of them
// are idle, so a warp does not wait for its longest ray; trav_step keeps the
// same node and triangle order as trace_closest / trace_any, so the answers
// are the same.
constexpr int kRefill = 8;

template <bool kAny, bool kCount>
__global__ void __launch_bounds__(128) k_trace(const WideNode *__restrict__ nodes, unsigned n_nodes,
                                               const float4 *__restrict__ tri, unsigned n_tris,
                                               const kgk_ray *__restrict__ rays, const float *__restrict__ tmax,
                                               int n, int32_t *id_out, float *t_out, uint8_t *occ,
                                               TraceCounters *ctr) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt = (1u << lane) - 1u;
    bool active = false, exhausted = false;
    int i = 0;
    unsigned done = 0;
    RayPre r;
    Trav c;
    TravStack stk;
    TravStats st{0, 0, 0};
    while (true) {
        const unsigned idle = __ballot_sync(~0u, !active);
        if (!exhausted && __popc(idle) >= kRefill) {
            int base = 0;
            if (lane == 0) base = (int)atomicAdd(&ctr->fetch, (unsigned long long)__popc(idle));
            base = __shfl_sync(~0u, base, 0);
            if (base + __popc(idle) >= n) exhausted = true;
            if (!active) {
                i = base + __popc(idle & lt);
                if (i < n) {
                    float3 o, d;
                    load_ray(rays, i, o, d);
                    r = make_ray(o, d);
                    trav_init(c, kAny && tmax ? tmax[i] : kBigT);
                    active = true;
                }
            }
        }
        if (!__any_sync(~0u, active)) break;
        if (active && trav_step<kCount>(nodes, n_nodes, tri, n_tris, r, c, stk, kAny, st)) {
            active = false;
            ++done;
            if (kAny) {
                occ[i] = c.hit_slot >= 0 ? 1 : 0;
            } else {
                id_out[i] = c.hit_slot >= 0 ? c.best_id : -1;
                t_out[i] = c.hit_slot >= 0 ? c.best_t : kBigT;
            }
        }
    }
    flush_counters(ctr, st.nodes, st.tris, st.overflow, done);
}

int grid_for(size_t n) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
    }
    return (int)std::min<size_t>((size_t)sms * 8, (n + 127) / 128);
}

}  // namespace

kgk_status trace_closest_dev(const DevScene &s, const kgk_ray *rays, size_t n, int32_t *id, float *t,
                             bool count, TraceCounters *ctr, cudaStream_t st) {
    if (n == 0) return KGK_OK;
    if (n > 0x7fffffff) return fail(KGK_ERR_INVALID_ARGUMENT, "trace: too many rays");
    const int g = grid_for(n);
    if (count)
        k_trace<false, true><<<g, 128, 0, st>>>(s.nodes, (unsigned)s.n_nodes, s.tri_rec, (unsigned)s.n_tris, rays,
                                                 nullptr, (int)n, id, t, nullptr, ctr);
    else
        k_trace<false, false><<<g, 128, 0, st>>>(s.nodes, (unsigned)s.n_nodes, s.tri_rec, (unsigned)s.n_tris, rays,
                                                  nullptr, (int)n, id, t, nullptr, ctr);
    KGK_CUDA(cudaGetLastError());
    return KGK_OK;
}

kgk_status trace_any_dev(const DevScene &s, const kgk_ray *rays, const float *tmax, size_t n, uint8_t *occ,
                         TraceCounters *ctr, cudaStream_t st) {
    if (n == 0) return KGK_OK;
    if (n > 0x7fffffff) return fail(KGK_ERR_INVALID_ARGUMENT, "trace: too many rays");
    k_trace<true, false><<<grid_for(n), 128, 0, st>>>(s.nodes, (unsigned)s.n_nodes, s.tri_rec, (unsigned)s.n_tris,
                                                       rays, tmax, (int)n, nullptr, nullptr, occ, ctr);
    KGK_CUDA(cudaGetLastError());
    return KGK_OK;
}

}  // namespace kgk
