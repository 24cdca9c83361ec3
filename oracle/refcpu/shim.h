/*
 * Force-included header that lets g++ compile the reference's CUDA C device
 * code as ordinary host C++ so the reference's own kernels can be executed on
 * the CPU as a parity oracle.  Kernel and device qualifiers become no-ops,
 * dynamic shared memory becomes thread-local storage (each OS thread runs one
 * emulated block at a time), and the built-in thread/block indices are
 * thread-local variables set by the launcher in launcher.cpp.
 *
 * Test infrastructure only: nothing in the product links this.
 */
#pragma once
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <math.h>
/* nvcc includes the runtime header implicitly; the stand-in is in stub_cuda/ */
#include <cuda_runtime.h>

#define __global__
#define __device__
#define __host__
#define __shared__ thread_local
#define __forceinline__ inline

struct refcpu_idx3 { unsigned int x, y, z; };
extern thread_local refcpu_idx3 threadIdx;
extern thread_local refcpu_idx3 blockIdx;
extern thread_local refcpu_idx3 blockDim;
extern thread_local refcpu_idx3 gridDim;
inline void __syncthreads() {}
