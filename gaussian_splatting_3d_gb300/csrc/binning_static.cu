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

// The array's device address belongs to one CUDA context: the runtime's
// primary context of a device, or a context the caller created and made
// current with the driver API, or the new primary context after a
// cudaDeviceReset.  Addresses are therefore cached per context, keyed by the
// context's unique id (cuCtxGetId: never reused within a process), not per
// device ordinal.  The two driver functions are reached through the
// runtime's entry-point query, so the library does not link libcuda.
using CtxGetCurrentFn = int (*)(void **ctx);
using CtxGetIdFn = int (*)(void *ctx, unsigned long long *id);

constexpr int kCacheSlots = 64;
struct ScratchSlot {
  unsigned long long ctx_id;
  void *addr;
};
std::mutex g_scratch_mutex;
ScratchSlot g_scratch_cache[kCacheSlots] = {};
int g_scratch_next = 0;  // round-robin replacement once every slot is used
bool g_driver_looked_up = false;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

void look_up_driver_functions() {
  if (g_driver_looked_up) return;
  g_driver_looked_up = true;
  cudaDriverEntryPointQueryResult q;
  void *f = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
          cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f);
  f = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
          cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f);
  cudaGetLastError();  // a failed query leaves no sticky runtime error behind
}

// Id of the context current on this thread; false if there is none (or the
// driver functions are unavailable).
bool current_context_id(unsigned long long *id) {
  if (!g_ctx_get_current || !g_ctx_get_id) return false;
  void *ctx = nullptr;
  if (g_ctx_get_current(&ctx) != 0 || ctx == nullptr) return false;
  return g_ctx_get_id(ctx, id) == 0;
}

// Device address of g_binning_scratch in the current context.  In host code
// the array's name is only a host-side stand-in, so the address must come
// from cudaGetSymbolAddress with the device (and context) current.  It is
// looked up once per context and cached; if the context cannot be
// identified, it is looked up on every call.
int scratch_address(void **out) {
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  look_up_driver_functions();
  unsigned long long id = 0;
  bool have_id = current_context_id(&id);
  if (have_id) {
    for (const ScratchSlot &s : g_scratch_cache)
      if (s.addr != nullptr && s.ctx_id == id) {
        *out = s.addr;
        return GSX_OK;
      }
  }
  void *p = nullptr;
  // also makes the device's primary context current if no context was
  cudaError_t e = cudaGetSymbolAddress(&p, g_binning_scratch);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(binning scratch)");
  if (!have_id) have_id = current_context_id(&id);
  if (have_id) {
    g_scratch_cache[g_scratch_next] = ScratchSlot{id, p};
    g_scratch_next = (g_scratch_next + 1) % kCacheSlots;
  }
  *out = p;
  return GSX_OK;
}

}  // namespace
}  // namespace gsx

using namespace gsx;

extern "C" int gsx_tile_culling_aabb_start_end_noalloc(
    int64_t n, int64_t n_keys, const int32_t *aabb_topleft, const int32_t *aabb_bottomright,
    const float *depth, int32_t n_tiles_h, int32_t n_tiles_w, int32_t *gaussian_ids,
    int32_t *start, int32_t *end, void *stream) {
  clear_error();
  int st = check_binning_sizes(n, n_keys, n_tiles_h, n_tiles_w);
  if (st != GSX_OK) return st;
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
  st = scratch_address(&scratch);
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
