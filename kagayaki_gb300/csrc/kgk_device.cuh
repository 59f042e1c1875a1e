// kgk_device.cuh - device helpers shared by the CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace kgk {

// ---- float3 arithmetic ---------------------------------------------------
__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 f3(float4 v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float3 &operator+=(float3 &a, float3 b) { a = a + b; return a; }
__device__ __forceinline__ float3 &operator*=(float3 &a, float3 b) { a = a * b; return a; }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float len3(float3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ float3 normalize3(float3 a) {
    float l = len3(a);
    return l > 0.0f ? a / l : f3(10000.0f, 0.0f, 0.0f);
}
__device__ __forceinline__ float3 fmin3(float3 a, float3 b) { return f3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
__device__ __forceinline__ float3 fmax3(float3 a, float3 b) { return f3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
__device__ __forceinline__ float comp(float3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
__device__ __forceinline__ float maxc(float3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
__device__ __forceinline__ float4 f4(float3 a, float w) { return make_float4(a.x, a.y, a.z, w); }

// ---- monotone float <-> int mapping for atomicMin / atomicMax ------------
__device__ __forceinline__ int f2o(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float o2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

// ---- scans ----------------------------------------------------------------
__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

// Exclusive scan over the block; `total` receives the block sum.  `ws` is a
// shared buffer of (blockDim.x / 32) ints.  All threads must call it.
__device__ __forceinline__ int block_excl_scan(int v, int *ws, int *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int inc = warp_incl_scan(v);
    if (lane == 31) ws[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        int w = lane < nw ? ws[lane] : 0;
        int wi = warp_incl_scan(w);
        if (lane < nw) ws[lane] = wi - w;
        if (lane == nw - 1) ws[31] = wi;  // requires nw <= 31 when read below
    }
    __syncthreads();
    int res = inc - v + ws[warp];
    int tot = ws[31];
    __syncthreads();
    if (total) *total = tot;
    return res;
}

__device__ __forceinline__ float surface_area(float3 lo, float3 hi) {
    float3 d = hi - lo;
    if (d.x < 0.0f || d.y < 0.0f || d.z < 0.0f) return 0.0f;
    return 2.0f * (d.x * d.y + d.y * d.z + d.z * d.x);
}

}  // namespace kgk
