// Shared definitions of the pump_gb300 CUDA sources.
//
// All translation units are compiled for sm_103a with -fmad=false: no
// multiply-add is contracted unless written as an explicit fma(), so every
// expression rounds exactly as the reference's C++ source does on a CPU.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pump.h"

namespace pump {

constexpr int kDim = 6;
constexpr int kThreads = 256;
constexpr int kNumSMs = 152;  // GB300: 2 dies x 76 SMs

// Records msg as this thread's last error; returns s.
pump_status_t set_error(pump_status_t s, const char *fmt, ...);
// Maps a CUDA error to PUMP_ERR_CUDA with its message; PUMP_OK on success.
pump_status_t cuda_status(cudaError_t e, const char *where);
// cuda_status(cudaGetLastError()) after a launch.
pump_status_t launch_status(const char *kernel);
// Stream-ordered allocation from the library's pool on the current device
// (freed with cudaFreeAsync); the pool keeps freed memory for reuse instead
// of returning it to the driver at every synchronisation.
cudaError_t pool_malloc_async(void **p, size_t bytes, cudaStream_t stream);
// Opts kernel fn in to `bytes` of dynamic shared memory on the current
// device.  The attribute is set only when the size grows, under a process-
// wide lock, so host threads that launch the same kernel at once never
// change it under one another's launches.
pump_status_t smem_attr(const void *fn, size_t bytes);

#define PUMP_CUDA_TRY(expr)                                     \
  do {                                                          \
    cudaError_t pump_ce_ = (expr);                                    \
    if (pump_ce_ != cudaSuccess) return ::pump::cuda_status(pump_ce_, #expr); \
  } while (0)
#define PUMP_TRY(expr)                  \
  do {                                  \
    pump_status_t pump_st_ = (expr);          \
    if (pump_st_ != PUMP_OK) return pump_st_;       \
  } while (0)

inline unsigned int grid_for(long long n, int threads) {
  long long g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  return (unsigned int)g;
}

// Order-preserving 32-bit keys of binary32 values (negative NaNs first,
// positive NaNs last), computed from the value's bits.  Keys are built from
// integer loads of the cost arrays and results stored as integers: a value
// that passes through a float register may come back with other NaN bits
// (code generated for a float load feeding a select turned positive NaNs
// into the key of -0.0).
__device__ __forceinline__ uint32_t key_of_bits(uint32_t u) {
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ uint32_t bits_of_key(uint32_t k) {
  return (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
}

// ---------------------------------------------------------------------------
// Integer powers of a float promoted to double, correctly rounded: the square
// of a float is exact in binary64, so each result below is rounded once.
// (The reference writes pow(float, int), promoted to pow(double, double).)
__host__ __device__ __forceinline__ double p2f(float x) { double d = x; return d * d; }
__host__ __device__ __forceinline__ double p3f(float x) { double d = x; return (d * d) * d; }
__host__ __device__ __forceinline__ double p4f(float x) { double d = x; double s = d * d; return s * s; }

// Block-wide contiguous copies between global and shared memory: 16-byte
// accesses when the global address and the count allow, so a block's
// per-thread records (strided, uncoalesced when each thread stores its own)
// move as whole 128-byte lines.  Callers synchronise around them.
__device__ __forceinline__ void block_store(float *__restrict__ dst, const float *src, int n) {
  if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0 && (n & 3) == 0) {
    float4 *d4 = reinterpret_cast<float4 *>(dst);
    const float4 *s4 = reinterpret_cast<const float4 *>(src);
    for (int i = threadIdx.x; i < n / 4; i += blockDim.x) d4[i] = s4[i];
  } else {
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
  }
}
__device__ __forceinline__ void block_load(float *dst, const float *__restrict__ src, int n) {
  if ((reinterpret_cast<uintptr_t>(src) & 15) == 0 && (n & 3) == 0) {
    float4 *d4 = reinterpret_cast<float4 *>(dst);
    const float4 *s4 = reinterpret_cast<const float4 *>(src);
    for (int i = threadIdx.x; i < n / 4; i += blockDim.x) d4[i] = __ldg(&s4[i]);
  } else {
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = __ldg(&src[i]);
  }
}

// `const float g = -9.81;` (2pBVP.cu:3)
#define PUMP_G ((float)-9.81)

}  // namespace pump
