/*
 * ref_shim.h -- test infrastructure only.
 *
 * Minimal host-side stand-ins for the CUDA language extensions used by the
 * reference kernels in mepgl/src/nlcg.cu and mepgl/src/interpolation.cu, so
 * that those __global__ functions compile unchanged as plain C++ and can be
 * driven serially on the CPU (see ref_driver.cpp).  Nothing here is shipped:
 * the product path never links this file.
 *
 * Each kernel launch is emulated by setting the thread-local index variables
 * below and calling the kernel body once per (block, thread).
 */
#pragma once

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline

struct dim3 {
    unsigned int x, y, z;
};

extern thread_local dim3 threadIdx;
extern thread_local dim3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

struct float2 { float x, y; };
struct float4 { float x, y, z, w; };
struct double2 { double x, y; };
struct double4 { double x, y, z, w; };

/* CUDA's overloaded max(): the kernels call it with mixed float/double. */
inline double max(double a, double b) { return a > b ? a : b; }
inline double max(double a, float b) { return max(a, (double)b); }
inline double max(float a, double b) { return max((double)a, b); }
inline float max(float a, float b) { return a > b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }

/* Serial emulation: one thread at a time, so a plain add is exact. */
inline float atomicAdd(float *p, float v) { float o = *p; *p = o + v; return o; }
inline double atomicAdd(double *p, double v) { double o = *p; *p = o + v; return o; }

inline void __syncthreads() {}

using std::pow;
using std::sqrt;
