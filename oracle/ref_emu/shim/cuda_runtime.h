// TEST INFRASTRUCTURE ONLY.  Host-compiler stand-in for the CUDA runtime
// header, so that the reference's kernel sources can be compiled by g++ and
// executed by the block/thread emulator in emu.h (one std::thread per CUDA
// thread, a condition-variable barrier for __syncthreads, std::atomic_ref
// compare-and-swap for atomicAdd).  Declares only what those sources use.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <math.h>

#define __host__
#define __device__
#define __global__
#define __forceinline__ inline
#define __shared__ static
#define __device_builtin__
#define __align__(n) alignas(n)

struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct alignas(16) float4 { float x, y, z, w; };
struct int2 { int x, y; };
struct int3 { int x, y, z; };
struct alignas(16) int4 { int x, y, z, w; };
struct uint2 { unsigned x, y; };
struct uint3 { unsigned x, y, z; };
struct uint4 { unsigned x, y, z, w; };
struct dim3 {
  unsigned x, y, z;
  dim3(unsigned x_ = 1, unsigned y_ = 1, unsigned z_ = 1) : x(x_), y(y_), z(z_) {}
};

inline float2 make_float2(float x, float y) { return {x, y}; }
inline float3 make_float3(float x, float y, float z) { return {x, y, z}; }
inline float4 make_float4(float x, float y, float z, float w) { return {x, y, z, w}; }
inline int2 make_int2(int x, int y) { return {x, y}; }
inline int3 make_int3(int x, int y, int z) { return {x, y, z}; }
inline int4 make_int4(int x, int y, int z, int w) { return {x, y, z, w}; }
inline uint2 make_uint2(unsigned x, unsigned y) { return {x, y}; }
inline uint3 make_uint3(unsigned x, unsigned y, unsigned z) { return {x, y, z}; }
inline uint4 make_uint4(unsigned x, unsigned y, unsigned z, unsigned w) { return {x, y, z, w}; }

// device-side math the sources use
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline unsigned int min(unsigned a, unsigned b) { return a < b ? a : b; }
inline unsigned int max(unsigned a, unsigned b) { return a > b ? a : b; }
inline float rsqrtf(float x) { return 1.0f / sqrtf(x); }
inline float __expf(float x) { return expf(x); }

#include "emu.h"

typedef int cudaError_t;
enum { cudaSuccess = 0 };
typedef void *cudaStream_t;
typedef void *cudaEvent_t;
enum cudaMemcpyKind { cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };

inline cudaError_t cudaMalloc(void **p, size_t n) {
  *p = std::malloc(n ? n : 1);
  return *p ? cudaSuccess : 2;
}
inline cudaError_t cudaFree(void *p) {
  std::free(p);
  return cudaSuccess;
}
inline cudaError_t cudaMemset(void *p, int v, size_t n) {
  std::memset(p, v, n);
  return cudaSuccess;
}
inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) {
  std::memmove(d, s, n);
  return cudaSuccess;
}
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline const char *cudaGetErrorString(cudaError_t) { return "emulated"; }
inline cudaError_t cudaEventCreate(cudaEvent_t *e) {
  *e = nullptr;
  return cudaSuccess;
}
inline cudaError_t cudaEventDestroy(cudaEvent_t) { return cudaSuccess; }
inline cudaError_t cudaEventRecord(cudaEvent_t, int) { return cudaSuccess; }
inline cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
inline cudaError_t cudaEventElapsedTime(float *ms, cudaEvent_t, cudaEvent_t) {
  *ms = 0.0f;
  return cudaSuccess;
}

template <typename T, typename U>
inline T emu_atomic_add_float(T *p, T v) {  // compare-and-swap on the bit pattern
  U *bits = reinterpret_cast<U *>(p);
  U old = __atomic_load_n(bits, __ATOMIC_RELAXED), want;
  T cur;
  do {
    std::memcpy(&cur, &old, sizeof(T));
    T next = cur + v;
    std::memcpy(&want, &next, sizeof(T));
  } while (!__atomic_compare_exchange_n(bits, &old, want, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED));
  return cur;
}
inline float atomicAdd(float *p, float v) { return emu_atomic_add_float<float, uint32_t>(p, v); }
inline double atomicAdd(double *p, double v) { return emu_atomic_add_float<double, uint64_t>(p, v); }
inline int atomicAdd(int *p, int v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }
inline unsigned atomicAdd(unsigned *p, unsigned v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }

// warp shuffles appear only in functions the emulated path never calls
float __shfl_xor_sync(unsigned mask, float v, int lane);
float __shfl_down_sync(unsigned mask, float v, int lane);
