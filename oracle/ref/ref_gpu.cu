/*
 * ref_gpu.cu - the reference's own render kernel (render.cuh:21-49, with
 * RayTrace and everything it calls) and its ApplySVGF kernel (SVGF.cuh:495-522)
 * compiled for sm_103a into a cubin, so that the reference's CUDA renderer and
 * denoiser can be timed on the GPU beside the new ones.  TEST AND MEASUREMENT INFRASTRUCTURE: oracle/Makefile (target
 * `refgpu`) builds it from the reference headers where they lie, with
 * ref_gpu_shim.h force-included; oracle/ref_gpu.py loads the cubin through
 * the CUDA driver API.  Nothing in the product links it.
 *
 * With KGK_REF_COUNT the traversal stack (struct_stack.cuh, a fixed-size
 * stack) is replaced by an equivalent class whose constructor counts one ray
 * per traversal call, the ray count of the reference's Mrays/s; the timed
 * cubin is built without it.
 */
#ifdef KGK_REF_COUNT
#define CUDA_MYPT_STRUCT_STACK_CUH
__device__ unsigned long long kgk_ref_traversals;
template <class T, int N> class stack {
    T buf[N];
    int idx;

public:
    __device__ stack() : idx(-1) { atomicAdd(&kgk_ref_traversals, 1ull); }
    __device__ T &top() { return buf[idx]; }
    __device__ void push(T const &v) { buf[++idx] = v; }
    __device__ T pop() { return buf[idx--]; }
    __device__ bool full() { return idx == (N - 1); }
    __device__ bool empty() { return idx == -1; }
};
#endif

#include "struct_Camera.cuh"
#include "struct_Xorshift.cuh"
#include "NextEventEstimation.cuh"
#include "render.cuh"
// ApplySVGF (SVGF.cuh:495-522), the kernel main.cu:160-166 launches on each
// rendered frame, timed beside the library's kgk_svgf_apply
#include "SVGF.cuh"
