// brdf.cu - kgk_disney_eval: the device's evaluation of the reference's
// Disney BRDF and its sampling pdf (evaluate_Disney_BRDF /
// evaluate_Disney_BRDF_pdf, Disney_BRDF.cuh:118-183) with the parameters
// RayTrace sets up (RayTrace.cuh:85-92): the functions the compat estimator
// calls, exposed so they can be compared with the reference's own values.
#include <algorithm>

#include "kgk_internal.h"
#include "shading.cuh"

namespace kgk {
namespace {

__global__ void k_disney_eval(kgk_material m, int n, const float *wo, const float *wi, const float *nrm,
                              float *brdf, float *pdf) {
    const DisneyParams p = disney_params(m);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float3 o = f3(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
        const float3 in = f3(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
        const float3 N = f3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
        float3 u, v, w;
        onb_ref(N, u, v, w);
        const float3 b = disney_eval<true>(m, p, o, in, N, u, v, w);
        brdf[3 * i] = b.x;
        brdf[3 * i + 1] = b.y;
        brdf[3 * i + 2] = b.z;
        pdf[i] = disney_pdf_ref(p, in, o, N, u, v, w);
    }
}

}  // namespace
}  // namespace kgk

extern "C" kgk_status kgk_disney_eval(const kgk_material *mat, int32_t n, const float *wo, const float *wi,
                                      const float *nrm, float *brdf, float *pdf) {
    using namespace kgk;
    if (!mat || !wo || !wi || !nrm || !brdf || !pdf || n < 0)
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_disney_eval: NULL argument or negative count");
    if (n == 0) return KGK_OK;
    const size_t v3 = (size_t)n * 3 * sizeof(float), v1 = (size_t)n * sizeof(float);
    float *d = nullptr;
    KGK_TRY(dmalloc((void **)&d, 4 * v3 + v1, "kgk_disney_eval buffers"));
    float *dwo = d, *dwi = d + 3 * (size_t)n, *dn = d + 6 * (size_t)n, *db = d + 9 * (size_t)n,
          *dp = d + 12 * (size_t)n;
    cudaError_t e = cudaMemcpy(dwo, wo, v3, cudaMemcpyDefault);
    if (e == cudaSuccess) e = cudaMemcpy(dwi, wi, v3, cudaMemcpyDefault);
    if (e == cudaSuccess) e = cudaMemcpy(dn, nrm, v3, cudaMemcpyDefault);
    if (e == cudaSuccess) {
        const int blocks = std::min((n + 255) / 256, 1024);
        k_disney_eval<<<blocks, 256>>>(*mat, n, dwo, dwi, dn, db, dp);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(brdf, db, v3, cudaMemcpyDefault);
    if (e == cudaSuccess) e = cudaMemcpy(pdf, dp, v1, cudaMemcpyDefault);
    dfree(d);
    if (e != cudaSuccess) return cuda_fail(e, "kgk_disney_eval");
    return KGK_OK;
}
