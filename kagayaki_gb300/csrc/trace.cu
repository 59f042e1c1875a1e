// trace.cu - batch closest-hit and occlusion queries (the parity entry
// points kgk_trace_closest / kgk_trace_any).  One thread per ray.
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

template <bool kCount>
__global__ void __launch_bounds__(128) k_trace_closest(const WideNode *__restrict__ nodes, unsigned n_nodes,
                                                       const float4 *__restrict__ tri, unsigned n_tris,
                                                       const kgk_ray *__restrict__ rays, int n,
                                                       int32_t *id_out, float *t_out,
                                                       TraceCounters *ctr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    TravStats st{0, 0, 0};
    if (i < n) {
        float3 o, d;
        load_ray(rays, i, o, d);
        const RayPre r = make_ray(o, d);
        float best_t = kBigT, u = 0.0f, v = 0.0f;
        int best_id = 0x7fffffff;
        int slot = trace_closest<kCount>(nodes, n_nodes, tri, n_tris, r, best_t, best_id, u, v, st);
        id_out[i] = slot >= 0 ? best_id : -1;
        t_out[i] = slot >= 0 ? best_t : kBigT;
    }
    flush_counters(ctr, st.nodes, st.tris, st.overflow, i < n ? 1u : 0u);
}

__global__ void __launch_bounds__(128) k_trace_any(const WideNode *__restrict__ nodes, unsigned n_nodes,
                                                   const float4 *__restrict__ tri, unsigned n_tris,
                                                   const kgk_ray *__restrict__ rays,
                                                   const float *__restrict__ tmax, int n,
                                                   uint8_t *occ, TraceCounters *ctr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    TravStats st{0, 0, 0};
    if (i < n) {
        float3 o, d;
        load_ray(rays, i, o, d);
        const RayPre r = make_ray(o, d);
        const float tm = tmax ? tmax[i] : kBigT;
        occ[i] = trace_any<false>(nodes, n_nodes, tri, n_tris, r, tm, st) ? 1 : 0;
    }
    flush_counters(ctr, st.nodes, st.tris, st.overflow, i < n ? 1u : 0u);
}

}  // namespace

kgk_status trace_closest_dev(const DevScene &s, const kgk_ray *rays, size_t n, int32_t *id, float *t,
                             bool count, TraceCounters *ctr, cudaStream_t st) {
    if (n == 0) return KGK_OK;
    if (n > 0x7fffffff) return fail(KGK_ERR_INVALID_ARGUMENT, "trace: too many rays");
    const int g = (int)((n + 127) / 128);
    if (count)
        k_trace_closest<true><<<g, 128, 0, st>>>(s.nodes, (unsigned)s.n_nodes, s.tri_rec, (unsigned)s.n_tris, rays, (int)n, id, t, ctr);
    else
        k_trace_closest<false><<<g, 128, 0, st>>>(s.nodes, (unsigned)s.n_nodes, s.tri_rec, (unsigned)s.n_tris, rays, (int)n, id, t, ctr);
    KGK_CUDA(cudaGetLastError());
    return KGK_OK;
}

kgk_status trace_any_dev(const DevScene &s, const kgk_ray *rays, const float *tmax, size_t n, uint8_t *occ,
                         TraceCounters *ctr, cudaStream_t st) {
    if (n == 0) return KGK_OK;
    if (n > 0x7fffffff) return fail(KGK_ERR_INVALID_ARGUMENT, "trace: too many rays");
    const int g = (int)((n + 127) / 128);
    k_trace_any<<<g, 128, 0, st>>>(s.nodes, (unsigned)s.n_nodes, s.tri_rec, (unsigned)s.n_tris, rays, tmax, (int)n, occ, ctr);
    KGK_CUDA(cudaGetLastError());
    return KGK_OK;
}

}  // namespace kgk
