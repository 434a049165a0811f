/* Host-C++ shim under which the reference's CUDA-C kernel text
 * (python/GPUFuncs_pycuda.py:7-1193, the string handed to pycuda's
 * SourceModule) compiles with g++ as ordinary functions.
 *
 * Test infrastructure: used only to build oracle/_ref/libctref.so, the
 * reference's own kernels run on the CPU as the timed CPU baseline and as a
 * cross-check of the oracle.  Each emulated CUDA thread is one call of the
 * kernel function with the per-OS-thread index variables below set by the
 * launcher (oracle/ref_launch.cpp).  atomicAdd becomes a plain add; the
 * launcher only runs threads that could race on one output element inside
 * one OS thread.
 */
#pragma once
#include <cmath>
#include <cstdio>
#include <algorithm>

struct ref_dim3 { unsigned x, y, z; };
extern thread_local ref_dim3 threadIdx, blockIdx, blockDim, gridDim;

#define __global__
#define __device__ static inline
#define __host__

static inline float atomicAdd(float *p, float v) { float o = *p; *p = o + v; return o; }
static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }
using std::fabs; using std::floor; using std::ceil; using std::sqrt; using std::cos; using std::sin;
using std::fmin; using std::fmax;
