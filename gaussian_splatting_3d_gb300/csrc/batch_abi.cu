// batch_abi.cu -- extern "C" entry points of the batched multi-view passes.
//
// Every stage of a batch of views is one launch: projection over all
// (view, Gaussian) items, one binning whose tile numbering is global over the
// batch, one raster launch over all tiles of all views, one projection
// backward.  Views may come from different scenes (forward) and may have
// different image sizes; they share the tile shape and the SH order.  The
// view table lives in device memory (caller-owned); the same table on the
// host gives the sizes, so no entry point reads device memory to plan.
#include <cstring>

#include <algorithm>

#include "gsx_internal.cuh"

using namespace gsx;

namespace {

struct BatchShape {
  int64_t n_items = 0, total_tiles = 0, max_n = 0;
  int32_t tile_w = 0, tile_h = 0, sh_order = 0, pixels_per_thread = 0;
  bool one_scene = true;
};

int check_views(const gsx_batch_view *hv, int32_t n_views, BatchShape &b) {
  if (!hv || n_views <= 0) {
    set_error("a batch needs a host copy of at least one view");
    return GSX_ERR_INVALID_ARG;
  }
  b.tile_w = hv[0].tile_w;
  b.tile_h = hv[0].tile_h;
  b.sh_order = hv[0].sh_order;
  b.pixels_per_thread = hv[0].pixels_per_thread;
  for (int32_t i = 0; i < n_views; ++i) {
    const gsx_batch_view &v = hv[i];
    if (v.tile_w != b.tile_w || v.tile_h != b.tile_h || v.sh_order != b.sh_order ||
        v.pixels_per_thread != hv[0].pixels_per_thread) {
      set_error("view %d: all views of a batch share the tile shape, SH order and raster schedule",
                i);
      return GSX_ERR_INVALID_ARG;
    }
    if (v.pixels_per_thread < 0 || v.pixels_per_thread > 2) {
      set_error("view %d: pixels_per_thread must be 0, 1 or 2 (got %d)", i, v.pixels_per_thread);
      return GSX_ERR_INVALID_ARG;
    }
    if (v.item_offset != b.n_items || v.tile_offset != b.total_tiles) {
      set_error("view %d: item_offset/tile_offset must be the running sums of the previous views", i);
      return GSX_ERR_INVALID_ARG;
    }
    if (v.n_gaussians < 0 || v.cam.width <= 0 || v.cam.height <= 0 || v.tile_w <= 0 ||
        v.tile_h <= 0 || v.tile_w * v.tile_h > 1024 || v.sh_order < 1 || v.sh_order > 4 ||
        v.sh_stride < v.sh_order * v.sh_order) {
      set_error("view %d: invalid sizes", i);
      return GSX_ERR_INVALID_ARG;
    }
    if ((int64_t)v.n_tiles_w * v.tile_w < v.cam.width ||
        (int64_t)v.n_tiles_h * v.tile_h < v.cam.height) {
      set_error("view %d: tile grid does not cover the image", i);
      return GSX_ERR_INVALID_ARG;
    }
    if (v.n_gaussians > 0 && (!v.mean || !v.qvec || !v.log_scale || !v.alpha_logit || !v.sh)) {
      set_error("view %d: null scene pointer", i);
      return GSX_ERR_INVALID_ARG;
    }
    if (((uintptr_t)v.qvec & 15) != 0) {
      set_error("view %d: qvec must be 16-byte aligned", i);
      return GSX_ERR_INVALID_ARG;
    }
    if (v.mean != hv[0].mean || v.n_gaussians != hv[0].n_gaussians) b.one_scene = false;
    b.n_items += v.n_gaussians;
    b.total_tiles += (int64_t)v.n_tiles_w * v.n_tiles_h;
    if (v.n_gaussians > b.max_n) b.max_n = v.n_gaussians;
  }
  if (b.n_items >= (int64_t(1) << 30) || b.total_tiles >= (int64_t(1) << 31)) {
    set_error("batch too large: %lld items, %lld tiles", (long long)b.n_items,
              (long long)b.total_tiles);
    return GSX_ERR_INVALID_ARG;
  }
  return GSX_OK;
}

RasterArgs batch_args(const gsx_batch_view *dv, int32_t n_views, const BatchShape &b,
                      int64_t key_capacity, const float *mean2d, const float *cov2d,
                      const float *alpha, const int32_t *start, const int32_t *end,
                      const int32_t *ids, float T_thresh) {
  RasterArgs a;
  std::memset(&a, 0, sizeof(a));
  a.n = b.n_items;
  a.n_keys = key_capacity;
  a.tile_w = b.tile_w;
  a.tile_h = b.tile_h;
  a.T_thresh = T_thresh;
  a.mean2d = mean2d;
  a.cov2d = cov2d;
  a.alpha = alpha;
  a.start = start;
  a.end = end;
  a.ids = ids;
  a.views = dv;
  a.n_views = n_views;
  a.pixels_per_thread = b.pixels_per_thread;
  return a;
}

inline cudaStream_t as_stream(void *s) { return static_cast<cudaStream_t>(s); }

}  // namespace

extern "C" {

size_t gsx_batch_view_size(void) { return sizeof(gsx_batch_view); }

int gsx_batch_project_forward(const gsx_batch_view *views_dev, const gsx_batch_view *views_host,
                              int32_t n_views, float frustum_radius, float tile_radius,
                              float *mean2d, float *cov2d, float *depth, float *alpha,
                              int32_t *rect, int32_t *counts, void *stream) {
  BatchShape b;
  int st = check_views(views_host, n_views, b);
  if (st != GSX_OK) return st;
  if (!views_dev || (b.n_items > 0 && (!mean2d || !cov2d || !depth || !alpha || !rect || !counts))) {
    set_error("null pointer argument");
    return GSX_ERR_INVALID_ARG;
  }
  return launch_project_forward_batch(views_dev, n_views, b.max_n, frustum_radius, tile_radius,
                                      mean2d, cov2d, depth, alpha, rect, counts,
                                      as_stream(stream));
}

int gsx_batch_bin_async(const gsx_batch_view *views_dev, const gsx_batch_view *views_host,
                        int32_t n_views, const int32_t *rect, const int32_t *counts,
                        const float *depth, int64_t key_capacity, int32_t *gaussian_ids,
                        int32_t *start, int32_t *end, void *workspace, size_t workspace_bytes,
                        void *stream) {
  BatchShape b;
  int st = check_views(views_host, n_views, b);
  if (st != GSX_OK) return st;
  if (key_capacity < 0 || key_capacity >= (int64_t(1) << 30)) {
    set_error("key capacity must be in [0, 2^30)");
    return GSX_ERR_INVALID_ARG;
  }
  if (!views_dev || !start || !end || (b.n_items > 0 && (!rect || !counts || !depth)) ||
      (key_capacity > 0 && !gaussian_ids)) {
    set_error("null pointer argument");
    return GSX_ERR_INVALID_ARG;
  }
  int64_t max_view_tiles = 0;  // the largest view's tile count: the width of the local tile ids
  for (int32_t i = 0; i < n_views; ++i)
    max_view_tiles = std::max(max_view_tiles, (int64_t)views_host[i].n_tiles_w * views_host[i].n_tiles_h);
  return run_binning_async(b.n_items, rect, rect + 2, 4, counts, depth, 0, 0, key_capacity,
                           gaussian_ids, start, end, workspace, workspace_bytes,
                           as_stream(stream), views_dev, n_views, b.total_tiles, max_view_tiles);
}

int gsx_batch_render_forward(const gsx_batch_view *views_dev, const gsx_batch_view *views_host,
                             int32_t n_views, int64_t key_capacity, const float *mean2d,
                             const float *cov2d, const float *alpha, const int32_t *start,
                             const int32_t *end, const int32_t *gaussian_ids, float T_thresh,
                             const int32_t *tile_order, uint32_t *work_counter, void *stream) {
  BatchShape b;
  int st = check_views(views_host, n_views, b);
  if (st != GSX_OK) return st;
  for (int32_t i = 0; i < n_views; ++i)
    if (!views_host[i].out) {
      set_error("view %d: null output image", i);
      return GSX_ERR_INVALID_ARG;
    }
  if (!views_dev || !start || !end || (key_capacity > 0 && !gaussian_ids) ||
      (b.n_items > 0 && (!mean2d || !cov2d || !alpha))) {
    set_error("null pointer argument");
    return GSX_ERR_INVALID_ARG;
  }
  RasterArgs a = batch_args(views_dev, n_views, b, key_capacity, mean2d, cov2d, alpha, start, end,
                            gaussian_ids, T_thresh);
  a.tile_order = tile_order;
  a.work_counter = work_counter;
  return launch_raster_forward_batch(a, b.sh_order, b.total_tiles, as_stream(stream));
}

int gsx_batch_render_backward(const gsx_batch_view *views_dev, const gsx_batch_view *views_host,
                              int32_t n_views, int64_t key_capacity, const float *mean2d,
                              const float *cov2d, const float *alpha, const int32_t *start,
                              const int32_t *end, const int32_t *gaussian_ids, float *g_mean2d,
                              float *g_cov2d, float *g_alpha, float T_thresh,
                              const int32_t *tile_order, uint32_t *work_counter, void *stream) {
  BatchShape b;
  int st = check_views(views_host, n_views, b);
  if (st != GSX_OK) return st;
  for (int32_t i = 0; i < n_views; ++i)
    if (!views_host[i].out || !views_host[i].grad_out || !views_host[i].g_sh) {
      set_error("view %d: null image, image gradient or SH gradient", i);
      return GSX_ERR_INVALID_ARG;
    }
  if (!views_dev || !start || !end || (key_capacity > 0 && !gaussian_ids) ||
      (b.n_items > 0 && (!mean2d || !cov2d || !alpha || !g_mean2d || !g_cov2d || !g_alpha))) {
    set_error("null pointer argument");
    return GSX_ERR_INVALID_ARG;
  }
  RasterArgs a = batch_args(views_dev, n_views, b, key_capacity, mean2d, cov2d, alpha, start, end,
                            gaussian_ids, T_thresh);
  a.g_mean2d = g_mean2d;
  a.g_cov2d = g_cov2d;
  a.g_alpha = g_alpha;
  a.tile_order = tile_order;
  a.work_counter = work_counter;
  return launch_raster_backward_batch(a, b.sh_order, b.total_tiles, as_stream(stream));
}

int gsx_batch_project_backward(const gsx_batch_view *views_dev, const gsx_batch_view *views_host,
                               int32_t n_views, const int32_t *counts, const float *g_mean2d,
                               const float *g_cov2d, const float *g_alpha, int32_t grad_flags,
                               void *stream) {
  if ((grad_flags & ~GSX_GRAD_EXACT) != 0) {
    set_error("unknown grad_flags bits 0x%x", grad_flags);
    return GSX_ERR_INVALID_ARG;
  }
  BatchShape b;
  int st = check_views(views_host, n_views, b);
  if (st != GSX_OK) return st;
  if (!b.one_scene) {
    set_error("the batched projection backward needs all views to share one scene");
    return GSX_ERR_INVALID_ARG;
  }
  const gsx_batch_view &v = views_host[0];
  if (!views_dev || (b.n_items > 0 && (!counts || !g_mean2d || !g_cov2d || !g_alpha ||
                                       !v.g_mean || !v.g_qvec || !v.g_log_scale ||
                                       !v.g_alpha_logit))) {
    set_error("null pointer argument");
    return GSX_ERR_INVALID_ARG;
  }
  if (((uintptr_t)v.g_qvec & 15) != 0 || ((uintptr_t)g_cov2d & 15) != 0 ||
      ((uintptr_t)g_mean2d & 7) != 0) {
    set_error("g_qvec and g_cov2d must be 16-byte aligned, g_mean2d 8-byte aligned");
    return GSX_ERR_INVALID_ARG;
  }
  return launch_project_backward_batch(views_dev, n_views, v.n_gaussians, counts, g_mean2d,
                                       g_cov2d, g_alpha, grad_flags, as_stream(stream));
}

}  // extern "C"
