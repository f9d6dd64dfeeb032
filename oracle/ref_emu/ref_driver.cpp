// TEST INFRASTRUCTURE ONLY.  Runs the reference's own CUDA kernels on the CPU.
//
// The kernel and device-function sources are the reference's, included from
// line ranges extracted verbatim at build time (oracle/build_ref.py writes
// them under oracle/_ref/src with #line directives pointing back at the
// original files); only the host launch sites (triple-chevron syntax, which a
// host compiler cannot parse) are replaced by the emu::launch calls below,
// which follow the reference's host functions step by step.
#include "cuda_runtime.h"

thread_local EmuIdx threadIdx;
EmuIdx blockIdx, blockDim, gridDim;

#include "common.h"
#include <cub/cub.cuh>
#include "data_spec.h"
#include "kernels.h"
#include "shencoder.h"
#include "ref_vol_render_helpers.inc"
#include "ref_vol_render_sh.inc"
#include "ref_aabb_culling.inc"
#include "ref_culling.inc"

static unsigned ceil_div(unsigned long long a, unsigned b) { return unsigned((a + b - 1) / b); }

extern "C" {

// gs/src/include/culling.h:22-34
void ref_cull(uint32_t N, float *mean, float *qvec, float *svec, float *normal, float *pts,
              bool *mask, float thresh) {
  float3 *mean_ = reinterpret_cast<float3 *>(mean);
  float4 *qvec_ = reinterpret_cast<float4 *>(qvec);
  float3 *svec_ = reinterpret_cast<float3 *>(svec);
  float3 *normal_ = reinterpret_cast<float3 *>(normal);
  float3 *pts_ = reinterpret_cast<float3 *>(pts);
  emu::launch(ceil_div(N, N_THREADS), 1, N_THREADS, 1, [&] {
    culling_gaussian_bsphere_kernel(N, mean_, qvec_, svec_, normal_, pts_, mask, thresh);
  });
}

// gs/src/include/aabb_culling.h:192-260 (returns the slot counter, which the
// reference asserts equals N_with_dub)
int ref_bin(uint32_t N, uint32_t N_with_dub, uint32_t n_tiles_h, uint32_t n_tiles_w,
            int *gaussian_ids, int *start, int *end, int *aabb_topleft, int *aabb_bottomright,
            float *depth) {
  int n_tiles = n_tiles_h * n_tiles_w;
  int64_t *tiledepth, *sorted_tiledepth;
  int *unsorted_gaussian_ids, *size;
  cudaMalloc((void **)&tiledepth, sizeof(int64_t) * N_with_dub);
  cudaMalloc((void **)&size, sizeof(int));
  cudaMemset(size, 0, sizeof(int));
  int *tile_ids = reinterpret_cast<int *>(tiledepth);
  float *tile_depth = reinterpret_cast<float *>(tiledepth);
  cudaMalloc((void **)&sorted_tiledepth, sizeof(int64_t) * N_with_dub);
  cudaMalloc((void **)&unsorted_gaussian_ids, sizeof(int) * N_with_dub);
  cudaMemset(tiledepth, 0, sizeof(int64_t) * N_with_dub);
  emu::launch(ceil_div(N, N_THREADS), 1, N_THREADS, 1, [&] {
    fill_tiledepth_aabb(N, N_with_dub, n_tiles_h, n_tiles_w, tile_ids, tile_depth,
                        unsorted_gaussian_ids, aabb_topleft, aabb_bottomright, depth, size);
  });
  int size_h = *size;
  void *d_temp_storage = NULL;
  size_t temp_storage_bytes = 0;
  cub::DeviceRadixSort::SortPairs(d_temp_storage, temp_storage_bytes, tiledepth, sorted_tiledepth,
                                  unsorted_gaussian_ids, gaussian_ids, N_with_dub);
  cudaMalloc((void **)&d_temp_storage, temp_storage_bytes);
  cub::DeviceRadixSort::SortPairs(d_temp_storage, temp_storage_bytes, tiledepth, sorted_tiledepth,
                                  unsorted_gaussian_ids, gaussian_ids, N_with_dub);
  cudaMemset(start, -1, sizeof(int) * n_tiles);
  cudaMemset(end, -1, sizeof(int) * n_tiles);
  int *sorted_tile_ids = reinterpret_cast<int *>(sorted_tiledepth);
  if (N_with_dub > 0) {
    emu::launch(ceil_div(N_with_dub, N_THREADS), 1, N_THREADS, 1,
                [&] { fill_start_aabb(N_with_dub, sorted_tile_ids, start); });
    emu::launch(ceil_div(N_with_dub, N_THREADS), 1, N_THREADS, 1,
                [&] { fill_end_aabb(N_with_dub, sorted_tile_ids, end); });
  }
  cudaFree(d_temp_storage);
  cudaFree(tiledepth);
  cudaFree(sorted_tiledepth);
  cudaFree(unsorted_gaussian_ids);
  cudaFree(size);
  return size_h;
}

// gs/src/include/vol_render_sh.h:250-266 with the template dispatch of
// gs/src/render.cu:506-543
void ref_render_fwd(uint32_t C, uint32_t N, uint32_t N_with_dub, float *mean, float *cov,
                    float *sh_coeffs, float *alpha, int *start, int *end, int *gaussian_ids,
                    float *out_rgb, float *topleft, float *c2w, uint32_t tile_size,
                    uint32_t n_tiles_h, uint32_t n_tiles_w, float pixel_size_x, float pixel_size_y,
                    uint32_t H, uint32_t W, float thresh) {
#define GSX_REF_FWD(CC)                                                                        \
  emu::launch(n_tiles_w, n_tiles_h, tile_size * tile_size, 1, [&] {                          \
    tile_based_vol_rendering_sh_entry<CC>(N, N_with_dub, mean, cov, sh_coeffs, alpha, start, \
                                          end, gaussian_ids, out_rgb, topleft, c2w,          \
                                          tile_size, n_tiles_h, n_tiles_w, pixel_size_x,     \
                                          pixel_size_y, H, W, thresh);                       \
  })
  switch (C) {
    case 1: GSX_REF_FWD(1); break;
    case 2: GSX_REF_FWD(2); break;
    case 3: GSX_REF_FWD(3); break;
    case 4: GSX_REF_FWD(4); break;
  }
#undef GSX_REF_FWD
}

// gs/src/include/vol_render_sh.h:457-480 with the dispatch of gs/src/render.cu:573-623
void ref_render_bwd(uint32_t C, uint32_t N, uint32_t N_with_dub, float *mean, float *cov,
                    float *sh_coeffs, float *alpha, int *start, int *end, int *gaussian_ids,
                    float *out_rgb, float *grad_mean, float *grad_cov, float *grad_sh_coeffs,
                    float *grad_alpha, float *grad_out_rgb, float *topleft, float *c2w,
                    uint32_t tile_size, uint32_t n_tiles_h, uint32_t n_tiles_w, float pixel_size_x,
                    float pixel_size_y, uint32_t H, uint32_t W, float thresh) {
#define GSX_REF_BWD(CC)                                                                          \
  emu::launch(n_tiles_w, n_tiles_h, tile_size * tile_size, 1, [&] {                            \
    tile_based_vol_rendering_backward_sh_entry<CC>(                                            \
        N, N_with_dub, mean, cov, sh_coeffs, alpha, start, end, gaussian_ids, out_rgb,         \
        grad_mean, grad_cov, grad_sh_coeffs, grad_alpha, grad_out_rgb, topleft, c2w, tile_size, \
        n_tiles_h, n_tiles_w, pixel_size_x, pixel_size_y, H, W, thresh);                       \
  })
  switch (C) {
    case 1: GSX_REF_BWD(1); break;
    case 2: GSX_REF_BWD(2); break;
    case 3: GSX_REF_BWD(3); break;
    case 4: GSX_REF_BWD(4); break;
  }
#undef GSX_REF_BWD
}

}  // extern "C"
