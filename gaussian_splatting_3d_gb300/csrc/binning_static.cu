// binning_static.cu -- tile binning for callers that cannot allocate device
// memory.
//
// Some hosts of this library may not call cudaMalloc at all: a renderer
// plugin living inside another application's fixed device-memory budget, a
// real-time loop that must never hit the allocator (a cudaMalloc can
// synchronise the device and stall every stream), or a runtime that forbids
// allocation after start-up.  They cannot provide the scratch workspace that
// gsx_tile_culling_aabb_start_end expects, so this file keeps one scratch
// array in the library's own static device memory and lends it to
// gsx_tile_culling_aabb_start_end_noalloc.
//
// The array is kStaticScratchBytes (64 MiB) per device; every GPU on which
// the library is loaded holds it until the process exits.  All calls share
// it and it keeps the previous call's contents (the binning clears the
// counters, histograms and look-back flags it needs at the start of every
// call), so calls that overlap on the GPU -- on different streams or from
// different host threads -- race on it and must be serialised by the caller.
#include <mutex>

#include "gsx_internal.cuh"

namespace gsx {
namespace {

constexpr size_t kStaticScratchBytes = size_t(64) << 20;

static __device__ __align__(256) unsigned char g_binning_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of g_binning_scratch on the current device, looked up once
// per device.  In host code the array's name is only a host-side stand-in,
// so the address must come from cudaGetSymbolAddress with the device current.
int scratch_address(void **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device ordinal %d is outside the supported range [0, %d)", dev, kMaxDevices);
    return GSX_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (g_scratch_addr[dev] == nullptr) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_binning_scratch);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(binning scratch)");
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return GSX_OK;
}

}  // namespace
}  // namespace gsx

using namespace gsx;

extern "C" int gsx_tile_culling_aabb_start_end_noalloc(
    int64_t n, int64_t n_keys, const int32_t *aabb_topleft, const int32_t *aabb_bottomright,
    const float *depth, int32_t n_tiles_h, int32_t n_tiles_w, int32_t *gaussian_ids,
    int32_t *start, int32_t *end, void *stream) {
  if (n < 0 || n >= (int64_t(1) << 30) || n_keys < 0 || n_keys >= (int64_t(1) << 30)) {
    set_error("n and n_keys must be in [0, 2^30) (got %lld, %lld)", (long long)n,
              (long long)n_keys);
    return GSX_ERR_INVALID_ARG;
  }
  if (n_tiles_h <= 0 || n_tiles_w <= 0 || (int64_t)n_tiles_h * n_tiles_w >= (int64_t(1) << 31)) {
    set_error("tile grid must be positive and below 2^31 tiles (got %d x %d)", n_tiles_w,
              n_tiles_h);
    return GSX_ERR_INVALID_ARG;
  }
  if (!start || !end || (n > 0 && (!aabb_topleft || !aabb_bottomright || !depth)) ||
      (n_keys > 0 && !gaussian_ids)) {
    set_error("null pointer argument");
    return GSX_ERR_INVALID_ARG;
  }
  const int64_t n_tiles = (int64_t)n_tiles_h * n_tiles_w;
  const size_t need = binning_workspace_bytes(n, n_keys, n_tiles);
  if (need > kStaticScratchBytes) {
    set_error(
        "%lld Gaussians with %lld keys need %zu bytes of scratch, more than the %zu-byte static "
        "array; use gsx_tile_culling_aabb_start_end with a caller-provided workspace",
        (long long)n, (long long)n_keys, need, kStaticScratchBytes);
    return GSX_ERR_CAPACITY;
  }
  void *scratch = nullptr;
  int st = scratch_address(&scratch);
  if (st != GSX_OK) return st;
  int64_t got = 0;
  st = run_binning(n, aabb_topleft, aabb_bottomright, 2, nullptr, depth, n_tiles_w, n_tiles_h,
                   n_keys, gaussian_ids, start, end, &got, scratch, kStaticScratchBytes,
                   static_cast<cudaStream_t>(stream));
  if (st == GSX_ERR_CAPACITY && got != n_keys) st = GSX_OK;  // reported as a mismatch below
  if (st != GSX_OK) return st;
  if (got != n_keys) {
    set_error("the rectangles hold %lld keys but gaussian_ids has %lld entries", (long long)got,
              (long long)n_keys);
    return GSX_ERR_MISMATCH;
  }
  return GSX_OK;
}
