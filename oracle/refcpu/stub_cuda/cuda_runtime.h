/*
 * Minimal stand-in for the CUDA runtime header used only when the reference's
 * files that mix host launch code with kernels are compiled as host C++ for
 * the CPU kernel library.  The host functions of those files are compiled but
 * never called from that library (the reference's host side runs from its own
 * nvcc host build linked against fake_cudart.cpp), so these are inert.
 */
#pragma once
#include <cstdlib>
#include <cstring>
typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1,
                      cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3 };
template <class T> inline cudaError_t cudaMalloc(T **p, size_t n) { *p = (T *)std::malloc(n); return 0; }
inline cudaError_t cudaFree(void *p) { std::free(p); return 0; }
inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) { std::memcpy(d, s, n); return 0; }
inline cudaError_t cudaDeviceSynchronize() { return 0; }
inline cudaError_t cudaPeekAtLastError() { return 0; }
inline const char *cudaGetErrorString(cudaError_t) { return "no error"; }
