/*
 * ref_shim.h - force-included when the reference's render-path headers are
 * compiled as host C++ (oracle/Makefile target `ref`).  TEST INFRASTRUCTURE:
 * it only lets the reference's own source run on the CPU as a checker.
 *
 * It maps the CUDA keywords to nothing, gives the CUDA vector types and launch
 * indices host definitions, routes __syncthreads() to a hook the driver may
 * bind to a std::barrier (the race-free reading of SVGF.cuh), and defines
 * free() away because ConstructBVH.cuh:365-366 frees two stack arrays.
 */
#pragma once

#include <algorithm>
#include <array>
#include <cassert>
#include <cctype>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#define __host__
#define __device__
#define __global__
#define __constant__
#define __forceinline__ inline

struct int2 { int x, y; };
struct float2 { float x, y; };
struct kgk_uint3_ { unsigned x = 0, y = 0, z = 0; };
extern thread_local kgk_uint3_ blockIdx, threadIdx, blockDim;

void __syncthreads();

using std::abs;
using std::asin;
using std::cos;
using std::exp;
using std::fabs;
using std::isfinite;
using std::log;
using std::max;
using std::min;
using std::pow;
using std::sin;
using std::sqrt;

enum cudaMemcpyKind { cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2,
                      cudaMemcpyDeviceToDevice = 3 };
template <class T> inline int cudaMalloc(T **p, size_t n) { *p = (T *)std::malloc(n); return 0; }
inline int cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) {
    std::memcpy(d, s, n); return 0; }
inline int cudaMemset(void *d, int v, size_t n) { std::memset(d, v, n); return 0; }

#define free(p) ((void)0)
