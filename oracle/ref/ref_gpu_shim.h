/*
 * ref_gpu_shim.h - force-included when the reference's render kernel is
 * compiled for the GPU (oracle/Makefile target `refgpu`).  TEST AND
 * MEASUREMENT INFRASTRUCTURE.
 *
 * The reference's traversal calls free() on its two stack arrays from device
 * code (ConstructBVH.cuh:365-366); the device heap's free() of a pointer it
 * did not allocate is undefined.  The system headers are included first, then
 * free(...) is defined to nothing, so those two calls compile to nothing and
 * the rest of the reference is unchanged.
 */
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
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

#define free(p) ((void)0)
