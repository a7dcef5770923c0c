/*
 * cuda.h -- a CPU stand-in for the CUDA built-ins used by the reference
 * kernels (3D/CUDA/CUDA_NBody/src/Kernels.cu), so that the reference's own
 * kernel source compiles with g++ and runs on the host.
 *
 * TEST INFRASTRUCTURE ONLY (oracle recipe).  Each CUDA thread is a
 * cooperative fiber; __syncthreads() and __all_sync() are barriers over the
 * live threads of the block, resolved by the scheduler in fiber.cpp.  Fibers
 * never preempt each other, so the atomics below are plain read-modify-writes.
 */
#ifndef NBX_REF_SHIM_CUDA_H
#define NBX_REF_SHIM_CUDA_H

#include <math.h>
#include <stdio.h>
#include <algorithm>

struct nbx_dim3 {
    unsigned x, y, z;
};

struct nbx_fiber;
extern nbx_fiber *nbx_cur_fiber;
extern nbx_dim3 nbx_block_idx, nbx_block_dim, nbx_grid_dim;
nbx_dim3 &nbx_thread_idx();

#define threadIdx (nbx_thread_idx())
#define blockIdx nbx_block_idx
#define blockDim nbx_block_dim
#define gridDim nbx_grid_dim

#define __global__
#define __device__
#define __host__
#define __shared__

void nbx_syncthreads();
int nbx_all_sync(int pred);

#define __syncthreads() nbx_syncthreads()
#define __all_sync(mask, pred) nbx_all_sync((pred) ? 1 : 0)
#define __activemask() 0xffffffffu
#define __threadfence() ((void)0)

inline int atomicCAS(int *a, int cmp, int val) { int o = *a; if (o == cmp) *a = val; return o; }
inline int atomicExch(int *a, int val) { int o = *a; *a = val; return o; }
inline int atomicAdd(int *a, int val) { int o = *a; *a = o + val; return o; }
inline float atomicAdd(float *a, float val) { float o = *a; *a = o + val; return o; }
inline float rsqrt(float r) { return 1.0f / sqrtf(r); }

using std::max;
using std::min;

#endif
