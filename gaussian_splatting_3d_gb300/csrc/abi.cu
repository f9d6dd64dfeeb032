// abi.cu -- the extern "C" entry points declared in include/gsx.h: argument
// validation, status codes and a per-thread error message.  No entry point
// exits the process or allocates device memory.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "gsx_internal.cuh"

namespace gsx {

namespace {
thread_local char g_err[512] = {0};
std::atomic<unsigned long long> g_launches{0};
}

void count_launches(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_status(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return GSX_OK;
  set_error("%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
  return GSX_ERR_CUDA;
}

void clear_error() { g_err[0] = 0; }

}  // namespace gsx

using namespace gsx;

#define GSX_REQUIRE(cond, ...)      \
  do {                              \
    if (!(cond)) {                  \
      set_error(__VA_ARGS__);       \
      return GSX_ERR_INVALID_ARG;   \
    }                               \
  } while (0)

static inline cudaStream_t as_stream(void *s) { return static_cast<cudaStream_t>(s); }

namespace gsx {
int check_binning_sizes(int64_t n, int64_t cap, int32_t nth, int32_t ntw) {
  GSX_REQUIRE(n >= 0 && n < (1ll << 30), "n must be in [0, 2^30) (got %lld)", (long long)n);
  GSX_REQUIRE(cap >= 0 && cap < (1ll << 30), "key count must be in [0, 2^30) (got %lld)",
              (long long)cap);
  GSX_REQUIRE(nth > 0 && ntw > 0, "tile grid must be positive (got %d x %d)", ntw, nth);
  GSX_REQUIRE((int64_t)nth * ntw < (1ll << 31), "too many tiles");
  return GSX_OK;
}
}  // namespace gsx

extern "C" {

const char *gsx_status_string(int status) {
  switch (status) {
    case GSX_OK: return "ok";
    case GSX_ERR_INVALID_ARG: return "invalid argument";
    case GSX_ERR_CAPACITY: return "capacity exceeded";
    case GSX_ERR_TIMEOUT: return "device wait timed out";
    case GSX_ERR_CUDA: return "CUDA error";
    case GSX_ERR_MISMATCH: return "size mismatch";
  }
  return "unknown status";
}

const char *gsx_last_error(void) { return g_err; }

int gsx_abi_version(void) { return GSX_ABI_VERSION; }

uint64_t gsx_kernel_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int gsx_culling_gaussian_bsphere(int64_t n, const float *mean, const float *qvec,
                                 const float *svec, const float *normal,
                                 const float *pts, uint8_t *mask, float thresh,
                                 void *stream) {
  (void)qvec;
  g_err[0] = 0;
  GSX_REQUIRE(n >= 0, "n must be >= 0 (got %lld)", (long long)n);
  if (n == 0) return GSX_OK;
  GSX_REQUIRE(mean && svec && normal && pts && mask, "null pointer argument");
  return launch_cull_bsphere(n, mean, svec, normal, pts, mask, thresh, as_stream(stream));
}

size_t gsx_binning_workspace_bytes(int64_t n_gaussians, int64_t key_capacity,
                                   int64_t n_tiles) {
  if (n_gaussians < 0 || key_capacity < 0 || n_tiles < 0) return 0;
  return binning_workspace_bytes(n_gaussians, key_capacity, n_tiles);
}

int gsx_tile_culling_aabb_start_end(int64_t n, int64_t n_keys,
                                    const int32_t *aabb_topleft,
                                    const int32_t *aabb_bottomright,
                                    const float *depth, int32_t n_tiles_h,
                                    int32_t n_tiles_w, int32_t *gaussian_ids,
                                    int32_t *start, int32_t *end, void *workspace,
                                    size_t workspace_bytes, void *stream) {
  g_err[0] = 0;
  int st = check_binning_sizes(n, n_keys, n_tiles_h, n_tiles_w);
  if (st != GSX_OK) return st;
  GSX_REQUIRE(start && end, "null start/end");
  GSX_REQUIRE(n == 0 || (aabb_topleft && aabb_bottomright && depth), "null input pointer");
  GSX_REQUIRE(n_keys == 0 || gaussian_ids, "null gaussian_ids");
  GSX_REQUIRE(workspace || workspace_bytes == 0, "null workspace");
  int64_t got = 0;
  st = run_binning(n, aabb_topleft, aabb_bottomright, 2, nullptr, depth, n_tiles_w, n_tiles_h,
                   n_keys, gaussian_ids, start, end, &got, workspace, workspace_bytes,
                   as_stream(stream));
  if (st == GSX_ERR_CAPACITY && got != n_keys) st = GSX_OK;  // reported below
  if (st != GSX_OK) return st;
  if (got != n_keys) {
    set_error("the rectangles hold %lld keys but gaussian_ids has %lld entries",
              (long long)got, (long long)n_keys);
    return GSX_ERR_MISMATCH;
  }
  return GSX_OK;
}

int gsx_bin_gaussians(int64_t n, const int32_t *rect, const int32_t *counts,
                      const float *depth, int32_t n_tiles_w, int32_t n_tiles_h,
                      int64_t key_capacity, int32_t *gaussian_ids, int32_t *start,
                      int32_t *end, int64_t *n_keys_out, void *workspace,
                      size_t workspace_bytes, void *stream) {
  g_err[0] = 0;
  int st = check_binning_sizes(n, key_capacity, n_tiles_h, n_tiles_w);
  if (st != GSX_OK) return st;
  GSX_REQUIRE(start && end && n_keys_out, "null output pointer");
  GSX_REQUIRE(n == 0 || (rect && counts && depth), "null input pointer");
  GSX_REQUIRE(key_capacity == 0 || gaussian_ids, "null gaussian_ids");
  return run_binning(n, rect, rect + 2, 4, counts, depth, n_tiles_w, n_tiles_h, key_capacity,
                     gaussian_ids, start, end, n_keys_out, workspace, workspace_bytes,
                     as_stream(stream));
}

int gsx_bin_gaussians_async(int64_t n, const int32_t *rect, const int32_t *counts,
                            const float *depth, int32_t n_tiles_w, int32_t n_tiles_h,
                            int64_t key_capacity, int32_t *gaussian_ids, int32_t *start,
                            int32_t *end, void *workspace, size_t workspace_bytes,
                            void *stream) {
  g_err[0] = 0;
  int st = check_binning_sizes(n, key_capacity, n_tiles_h, n_tiles_w);
  if (st != GSX_OK) return st;
  GSX_REQUIRE(start && end, "null output pointer");
  GSX_REQUIRE(n == 0 || (rect && counts && depth), "null input pointer");
  GSX_REQUIRE(key_capacity == 0 || gaussian_ids, "null gaussian_ids");
  return run_binning_async(n, rect, rect + 2, 4, counts, depth, n_tiles_w, n_tiles_h,
                           key_capacity, gaussian_ids, start, end, workspace, workspace_bytes,
                           as_stream(stream));
}

size_t gsx_look_back_selftest_bytes(void) { return look_back_selftest_bytes(); }

int gsx_look_back_selftest(void *scratch, size_t scratch_bytes, uint32_t *error_bits, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(scratch, "null scratch");
  return look_back_selftest(scratch, scratch_bytes, error_bits, as_stream(stream));
}

int gsx_binning_status(const void *workspace, int64_t n_gaussians, int64_t key_capacity,
                       int32_t n_tiles_w, int32_t n_tiles_h, int64_t *n_keys_out,
                       void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(workspace, "null workspace");
  GSX_REQUIRE(n_gaussians >= 0 && key_capacity >= 0, "negative size");
  return binning_status(workspace, n_gaussians, key_capacity, n_tiles_w, n_tiles_h, n_keys_out,
                        nullptr, as_stream(stream));
}

int gsx_binning_status_copy_async(const void *workspace, int64_t n_gaussians,
                                  int64_t key_capacity, void *dst, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(workspace && dst, "null pointer argument");
  GSX_REQUIRE(n_gaussians >= 0 && key_capacity >= 0, "negative size");
  return copy_binning_status_async(workspace, n_gaussians, key_capacity, dst, as_stream(stream));
}

int gsx_binning_status_decode(const void *block, int64_t key_capacity, int32_t n_tiles_w,
                              int32_t n_tiles_h, int64_t *n_keys_out) {
  g_err[0] = 0;
  GSX_REQUIRE(block, "null status block");
  uint64_t w[2];
  std::memcpy(w, block, sizeof(w));
  if (n_keys_out) *n_keys_out = (int64_t)w[0];
  return decode_binning_status(w[0], (uint32_t)(w[1] & 0xffffffffu), key_capacity, n_tiles_w,
                               n_tiles_h);
}

static int check_raster(const RasterArgs &a, int C, int64_t n, int64_t n_keys) {
  GSX_REQUIRE(C >= 1 && C <= 4, "SH order C must be 1..4 (got %d)", C);
  GSX_REQUIRE(a.tile_w > 0 && a.tile_h > 0 && a.tile_w * a.tile_h <= 1024,
              "tile must have 1..1024 pixels (got %d x %d)", a.tile_w, a.tile_h);
  GSX_REQUIRE(a.width > 0 && a.height > 0, "image size must be positive");
  GSX_REQUIRE((int64_t)a.n_tiles_w * a.tile_w >= a.width &&
                  (int64_t)a.n_tiles_h * a.tile_h >= a.height,
              "tile grid %d x %d of %d x %d tiles does not cover %d x %d", a.n_tiles_w,
              a.n_tiles_h, a.tile_w, a.tile_h, a.width, a.height);
  GSX_REQUIRE(a.sh_stride >= C * C, "sh_stride %d < C*C", a.sh_stride);
  GSX_REQUIRE(a.pixels_per_thread >= 0 && a.pixels_per_thread <= 2,
              "pixels_per_thread must be 0, 1 or 2 (got %d)", a.pixels_per_thread);
  GSX_REQUIRE(n >= 0 && n_keys >= 0, "negative size");
  GSX_REQUIRE(a.start && a.end && a.topleft && a.c2w && a.out, "null pointer argument");
  GSX_REQUIRE(n_keys == 0 || a.ids, "null gaussian_ids");
  GSX_REQUIRE(n == 0 || (a.mean2d && a.cov2d && a.sh && a.alpha), "null Gaussian data");
  return GSX_OK;
}

static RasterArgs make_args(int64_t tile_w, int64_t tile_h, uint32_t ntw, uint32_t nth,
                            float psx, float psy, uint32_t H, uint32_t W, float thresh) {
  RasterArgs a;
  std::memset(&a, 0, sizeof(a));
  a.width = (int32_t)W;
  a.height = (int32_t)H;
  a.tile_w = (int32_t)tile_w;
  a.tile_h = (int32_t)tile_h;
  a.n_tiles_w = (int32_t)ntw;
  a.n_tiles_h = (int32_t)nth;
  a.psx = psx;
  a.psy = psy;
  a.T_thresh = thresh;
  return a;
}

int gsx_tile_based_vol_rendering_sh(
    int64_t n, int64_t n_keys, const float *mean, const float *cov,
    const float *sh_coeffs, const float *alpha, const int32_t *start,
    const int32_t *end, const int32_t *gaussian_ids, float *out,
    const float *topleft, const float *c2w, uint32_t tile_size,
    uint32_t n_tiles_h, uint32_t n_tiles_w, float pixel_size_x,
    float pixel_size_y, uint32_t H, uint32_t W, uint32_t C, float thresh,
    void *stream) {
  g_err[0] = 0;
  RasterArgs a = make_args(tile_size, tile_size, n_tiles_w, n_tiles_h, pixel_size_x,
                           pixel_size_y, H, W, thresh);
  a.sh_stride = (int32_t)(C * C);
  a.mean2d = mean;
  a.cov2d = cov;
  a.sh = sh_coeffs;
  a.alpha = alpha;
  a.start = start;
  a.end = end;
  a.ids = gaussian_ids;
  a.topleft = topleft;
  a.c2w = c2w;
  a.out = out;
  a.write_empty = 0;
  a.n = n;
  a.n_keys = n_keys;
  int st = check_raster(a, (int)C, n, n_keys);
  if (st != GSX_OK) return st;
  return launch_raster_forward(a, (int)C, as_stream(stream));
}

int gsx_tile_based_vol_rendering_backward_sh(
    int64_t n, int64_t n_keys, const float *mean, const float *cov,
    const float *sh_coeffs, const float *alpha, const int32_t *start,
    const int32_t *end, const int32_t *gaussian_ids, const float *out,
    float *grad_mean, float *grad_cov, float *grad_sh_coeffs, float *grad_alpha,
    const float *grad_out, const float *topleft, const float *c2w,
    uint32_t tile_size, uint32_t n_tiles_h, uint32_t n_tiles_w,
    float pixel_size_x, float pixel_size_y, uint32_t H, uint32_t W, uint32_t C,
    float thresh, void *stream) {
  g_err[0] = 0;
  RasterArgs a = make_args(tile_size, tile_size, n_tiles_w, n_tiles_h, pixel_size_x,
                           pixel_size_y, H, W, thresh);
  a.sh_stride = (int32_t)(C * C);
  a.mean2d = mean;
  a.cov2d = cov;
  a.sh = sh_coeffs;
  a.alpha = alpha;
  a.start = start;
  a.end = end;
  a.ids = gaussian_ids;
  a.topleft = topleft;
  a.c2w = c2w;
  a.out = const_cast<float *>(out);
  a.final_img = out;
  a.grad_out = grad_out;
  a.g_mean2d = grad_mean;
  a.g_cov2d = grad_cov;
  a.g_sh = grad_sh_coeffs;
  a.g_alpha = grad_alpha;
  a.n = n;
  a.n_keys = n_keys;
  int st = check_raster(a, (int)C, n, n_keys);
  if (st != GSX_OK) return st;
  GSX_REQUIRE(grad_out && (n == 0 || (grad_mean && grad_cov && grad_sh_coeffs && grad_alpha)),
              "null gradient pointer");
  return launch_raster_backward(a, (int)C, as_stream(stream));
}

int gsx_project_forward(int64_t n, const float *mean, const float *qvec,
                        const float *log_scale, const float *alpha_logit,
                        const gsx_camera *cam, float frustum_radius,
                        float tile_radius, int32_t tile_w, int32_t tile_h,
                        int32_t scales_are_activated, float *mean2d, float *cov2d,
                        float *depth, float *alpha, int32_t *rect,
                        int32_t *counts, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(n >= 0, "n must be >= 0");
  GSX_REQUIRE(cam, "null camera");
  GSX_REQUIRE(tile_w > 0 && tile_h > 0, "tile size must be positive");
  GSX_REQUIRE(cam->width > 0 && cam->height > 0, "image size must be positive");
  if (n == 0) return GSX_OK;
  GSX_REQUIRE(mean && qvec && log_scale && mean2d && cov2d && depth && alpha && rect && counts,
              "null pointer argument");
  GSX_REQUIRE(((uintptr_t)qvec & 15) == 0 && ((uintptr_t)cov2d & 15) == 0 &&
                  ((uintptr_t)rect & 15) == 0 && ((uintptr_t)mean2d & 7) == 0,
              "qvec, cov2d and rect must be 16-byte aligned, mean2d 8-byte aligned");
  return launch_project_forward(n, mean, qvec, log_scale, alpha_logit, *cam, frustum_radius,
                                tile_radius, tile_w, tile_h, scales_are_activated, mean2d,
                                cov2d, depth, alpha, rect, counts, as_stream(stream));
}

static int render_forward(const gsx_raster_params *p, int64_t n, int64_t n_keys,
                          const float *mean2d, const float *cov2d, const float *sh,
                          const float *alpha, const int32_t *start, const int32_t *end,
                          const int32_t *gaussian_ids, const float *topleft, const float *c2w,
                          float *out, const float *bg_rgb, const float *depth, float *alpha_out,
                          float *depth_out, const int32_t *tile_order, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(p, "null params");
  RasterArgs a = make_args(p->tile_w, p->tile_h, (uint32_t)p->n_tiles_w,
                           (uint32_t)p->n_tiles_h, p->pixel_size_x, p->pixel_size_y,
                           (uint32_t)p->height, (uint32_t)p->width, p->T_thresh);
  a.pixels_per_thread = p->pixels_per_thread;
  a.sh_stride = p->sh_stride;
  a.mean2d = mean2d;
  a.cov2d = cov2d;
  a.sh = sh;
  a.alpha = alpha;
  a.start = start;
  a.end = end;
  a.ids = gaussian_ids;
  a.topleft = topleft;
  a.c2w = c2w;
  a.out = out;
  a.write_empty = p->write_empty_tiles;
  a.n = n;
  a.n_keys = n_keys;
  if (bg_rgb) {
    a.has_bg = 1;
    a.bg[0] = bg_rgb[0];
    a.bg[1] = bg_rgb[1];
    a.bg[2] = bg_rgb[2];
  }
  GSX_REQUIRE(!depth_out || n == 0 || depth, "a depth map needs the per-Gaussian depth");
  a.depth = depth;
  a.alpha_out = alpha_out;
  a.depth_out = depth_out;
  a.tile_order = tile_order;
  int st = check_raster(a, p->sh_order, n, n_keys);
  if (st != GSX_OK) return st;
  return launch_raster_forward(a, p->sh_order, as_stream(stream));
}

int gsx_render_forward_maps(const gsx_raster_params *p, int64_t n, int64_t n_keys,
                            const float *mean2d, const float *cov2d, const float *sh,
                            const float *alpha, const int32_t *start, const int32_t *end,
                            const int32_t *gaussian_ids, const float *topleft, const float *c2w,
                            float *out, const float *bg_rgb, const float *depth,
                            float *alpha_out, float *depth_out, void *stream) {
  return render_forward(p, n, n_keys, mean2d, cov2d, sh, alpha, start, end, gaussian_ids, topleft,
                        c2w, out, bg_rgb, depth, alpha_out, depth_out, nullptr, stream);
}

int gsx_render_forward_ordered(const gsx_raster_params *p, int64_t n, int64_t n_keys,
                               const float *mean2d, const float *cov2d, const float *sh,
                               const float *alpha, const int32_t *start, const int32_t *end,
                               const int32_t *gaussian_ids, const float *topleft,
                               const float *c2w, float *out, const int32_t *tile_order,
                               void *stream) {
  if (!tile_order) {
    g_err[0] = 0;
    set_error("null tile_order");
    return GSX_ERR_INVALID_ARG;
  }
  return render_forward(p, n, n_keys, mean2d, cov2d, sh, alpha, start, end, gaussian_ids, topleft,
                        c2w, out, nullptr, nullptr, nullptr, nullptr, tile_order, stream);
}

int gsx_render_forward_rgb(const gsx_raster_params *p, int64_t n, int64_t n_keys,
                           const float *mean2d, const float *cov2d, const float *rgb,
                           const float *alpha, const int32_t *start, const int32_t *end,
                           const int32_t *gaussian_ids, const float *topleft, const float *c2w,
                           float *out, const int32_t *tile_order, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(p, "null params");
  RasterArgs a = make_args(p->tile_w, p->tile_h, (uint32_t)p->n_tiles_w,
                           (uint32_t)p->n_tiles_h, p->pixel_size_x, p->pixel_size_y,
                           (uint32_t)p->height, (uint32_t)p->width, p->T_thresh);
  a.pixels_per_thread = p->pixels_per_thread;
  a.sh_stride = 1;  // rgb [n,3] as one coefficient per channel
  a.mean2d = mean2d;
  a.cov2d = cov2d;
  a.sh = rgb;
  a.alpha = alpha;
  a.start = start;
  a.end = end;
  a.ids = gaussian_ids;
  a.topleft = topleft;
  a.c2w = c2w;
  a.out = out;
  a.write_empty = p->write_empty_tiles;
  a.n = n;
  a.n_keys = n_keys;
  a.tile_order = tile_order;
  int st = check_raster(a, 1, n, n_keys);
  if (st != GSX_OK) return st;
  return launch_raster_forward_rgb(a, as_stream(stream));
}

int gsx_render_backward_rgb(const gsx_raster_params *p, int64_t n, int64_t n_keys,
                            const float *mean2d, const float *cov2d, const float *rgb,
                            const float *alpha, const int32_t *start, const int32_t *end,
                            const int32_t *gaussian_ids, const float *topleft, const float *c2w,
                            const float *out, const float *grad_out, float *grad_mean2d,
                            float *grad_cov2d, float *grad_rgb, float *grad_alpha,
                            const int32_t *tile_order, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(p, "null params");
  RasterArgs a = make_args(p->tile_w, p->tile_h, (uint32_t)p->n_tiles_w,
                           (uint32_t)p->n_tiles_h, p->pixel_size_x, p->pixel_size_y,
                           (uint32_t)p->height, (uint32_t)p->width, p->T_thresh);
  a.pixels_per_thread = p->pixels_per_thread;
  a.sh_stride = 1;
  a.mean2d = mean2d;
  a.cov2d = cov2d;
  a.sh = rgb;
  a.alpha = alpha;
  a.start = start;
  a.end = end;
  a.ids = gaussian_ids;
  a.topleft = topleft;
  a.c2w = c2w;
  a.out = const_cast<float *>(out);
  a.final_img = out;
  a.grad_out = grad_out;
  a.g_mean2d = grad_mean2d;
  a.g_cov2d = grad_cov2d;
  a.g_sh = grad_rgb;
  a.g_alpha = grad_alpha;
  a.n = n;
  a.n_keys = n_keys;
  a.tile_order = tile_order;
  int st = check_raster(a, 1, n, n_keys);
  if (st != GSX_OK) return st;
  GSX_REQUIRE(grad_out && (n == 0 || (grad_mean2d && grad_cov2d && grad_rgb && grad_alpha)),
              "null gradient pointer");
  return launch_raster_backward_rgb(a, as_stream(stream));
}

int gsx_project_colors(int64_t n, const float *mean, const float *sh, int32_t sh_stride,
                       int32_t sh_order, const float *cam_pos, const int32_t *counts, float *rgb,
                       void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(n >= 0, "n must be >= 0 (got %lld)", (long long)n);
  if (n == 0) return GSX_OK;
  GSX_REQUIRE(mean && sh && cam_pos && rgb, "null pointer argument");
  GSX_REQUIRE(sh_order >= 1 && sh_order <= 4, "SH order C must be 1..4 (got %d)", sh_order);
  GSX_REQUIRE(sh_stride >= sh_order * sh_order, "sh_stride %d < C*C = %d", sh_stride,
              sh_order * sh_order);
  return launch_colors_forward(n, mean, sh, sh_stride, sh_order, cam_pos, counts, rgb,
                               as_stream(stream));
}

int gsx_project_colors_backward(int64_t n, const float *mean, const float *sh, int32_t sh_stride,
                                int32_t sh_order, const float *cam_pos, const int32_t *counts,
                                const float *rgb, const float *grad_rgb, float *grad_sh,
                                float *grad_mean, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(n >= 0, "n must be >= 0 (got %lld)", (long long)n);
  if (n == 0) return GSX_OK;
  GSX_REQUIRE(mean && sh && cam_pos && rgb && grad_rgb && grad_sh && grad_mean,
              "null pointer argument");
  GSX_REQUIRE(sh_order >= 1 && sh_order <= 4, "SH order C must be 1..4 (got %d)", sh_order);
  GSX_REQUIRE(sh_stride >= sh_order * sh_order, "sh_stride %d < C*C = %d", sh_stride,
              sh_order * sh_order);
  return launch_colors_backward(n, mean, sh, sh_stride, sh_order, cam_pos, counts, rgb, grad_rgb,
                                grad_sh, grad_mean, as_stream(stream));
}

int gsx_tile_order(const int32_t *start, const int32_t *end, int32_t n_tiles, int32_t *tile_order,
                   void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(n_tiles >= 0, "n_tiles must be >= 0 (got %d)", n_tiles);
  if (n_tiles == 0) return GSX_OK;
  GSX_REQUIRE(start && end && tile_order, "null pointer argument");
  return launch_tile_order(start, end, n_tiles, tile_order, as_stream(stream));
}

int gsx_render_forward(const gsx_raster_params *p, int64_t n, int64_t n_keys,
                       const float *mean2d, const float *cov2d, const float *sh,
                       const float *alpha, const int32_t *start, const int32_t *end,
                       const int32_t *gaussian_ids, const float *topleft,
                       const float *c2w, float *out, void *stream) {
  return gsx_render_forward_maps(p, n, n_keys, mean2d, cov2d, sh, alpha, start, end, gaussian_ids,
                                 topleft, c2w, out, nullptr, nullptr, nullptr, nullptr, stream);
}

static int render_backward(const gsx_raster_params *p, int64_t n, int64_t n_keys,
                           const float *mean2d, const float *cov2d, const float *sh,
                           const float *alpha, const int32_t *start, const int32_t *end,
                           const int32_t *gaussian_ids, const float *topleft, const float *c2w,
                           const float *out, const float *grad_out, float *grad_mean2d,
                           float *grad_cov2d, float *grad_sh, float *grad_alpha,
                           const int32_t *tile_order, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(p, "null params");
  RasterArgs a = make_args(p->tile_w, p->tile_h, (uint32_t)p->n_tiles_w,
                           (uint32_t)p->n_tiles_h, p->pixel_size_x, p->pixel_size_y,
                           (uint32_t)p->height, (uint32_t)p->width, p->T_thresh);
  a.pixels_per_thread = p->pixels_per_thread;
  a.sh_stride = p->sh_stride;
  a.mean2d = mean2d;
  a.cov2d = cov2d;
  a.sh = sh;
  a.alpha = alpha;
  a.start = start;
  a.end = end;
  a.ids = gaussian_ids;
  a.topleft = topleft;
  a.c2w = c2w;
  a.out = const_cast<float *>(out);
  a.final_img = out;
  a.grad_out = grad_out;
  a.g_mean2d = grad_mean2d;
  a.g_cov2d = grad_cov2d;
  a.g_sh = grad_sh;
  a.g_alpha = grad_alpha;
  a.n = n;
  a.n_keys = n_keys;
  int st = check_raster(a, p->sh_order, n, n_keys);
  if (st != GSX_OK) return st;
  GSX_REQUIRE(grad_out && (n == 0 || (grad_mean2d && grad_cov2d && grad_sh && grad_alpha)),
              "null gradient pointer");
  a.tile_order = tile_order;
  return launch_raster_backward(a, p->sh_order, as_stream(stream));
}

int gsx_render_backward(const gsx_raster_params *p, int64_t n, int64_t n_keys,
                        const float *mean2d, const float *cov2d, const float *sh,
                        const float *alpha, const int32_t *start,
                        const int32_t *end, const int32_t *gaussian_ids,
                        const float *topleft, const float *c2w, const float *out,
                        const float *grad_out, float *grad_mean2d,
                        float *grad_cov2d, float *grad_sh, float *grad_alpha,
                        void *stream) {
  return render_backward(p, n, n_keys, mean2d, cov2d, sh, alpha, start, end, gaussian_ids,
                         topleft, c2w, out, grad_out, grad_mean2d, grad_cov2d, grad_sh,
                         grad_alpha, nullptr, stream);
}

int gsx_render_backward_ordered(const gsx_raster_params *p, int64_t n, int64_t n_keys,
                                const float *mean2d, const float *cov2d, const float *sh,
                                const float *alpha, const int32_t *start, const int32_t *end,
                                const int32_t *gaussian_ids, const float *topleft,
                                const float *c2w, const float *out, const float *grad_out,
                                float *grad_mean2d, float *grad_cov2d, float *grad_sh,
                                float *grad_alpha, const int32_t *tile_order, void *stream) {
  if (!tile_order) {
    g_err[0] = 0;
    set_error("null tile_order");
    return GSX_ERR_INVALID_ARG;
  }
  return render_backward(p, n, n_keys, mean2d, cov2d, sh, alpha, start, end, gaussian_ids,
                         topleft, c2w, out, grad_out, grad_mean2d, grad_cov2d, grad_sh,
                         grad_alpha, tile_order, stream);
}

int gsx_raster_wait_selftest(uint32_t limit, uint32_t *polls_dev, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(polls_dev, "null polls pointer");
  GSX_REQUIRE(limit >= 1 && limit <= (1u << 20), "limit must be in [1, 2^20] (got %u)", limit);
  return raster_wait_selftest(limit, polls_dev, as_stream(stream));
}

int gsx_exp_selftest(const float *x, int64_t n, float *out, int32_t variant, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(n >= 0, "n must be >= 0");
  GSX_REQUIRE(n == 0 || (x && out), "null input or output");
  GSX_REQUIRE(variant >= 0 && variant <= 2, "variant must be 0, 1 or 2 (got %d)", variant);
  return exp_selftest(x, n, out, variant, as_stream(stream));
}

int gsx_raster_status(uint32_t *flags, int32_t clear, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(flags, "null flags pointer");
  return raster_status(flags, clear, as_stream(stream));
}

int gsx_project_backward(int64_t n, const float *mean, const float *qvec,
                         const float *log_scale, const float *alpha_logit,
                         const gsx_camera *cam, const int32_t *counts,
                         const float *grad_mean2d, const float *grad_cov2d,
                         const float *grad_alpha, float *grad_mean,
                         float *grad_qvec, float *grad_log_scale,
                         float *grad_alpha_logit, int32_t grad_flags, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(n >= 0, "n must be >= 0");
  GSX_REQUIRE(cam, "null camera");
  GSX_REQUIRE((grad_flags & ~GSX_GRAD_EXACT) == 0, "unknown grad_flags bits 0x%x", grad_flags);
  if (n == 0) return GSX_OK;
  GSX_REQUIRE(mean && qvec && log_scale && alpha_logit && counts && grad_mean2d &&
                  grad_cov2d && grad_alpha && grad_mean && grad_qvec && grad_log_scale &&
                  grad_alpha_logit,
              "null pointer argument");
  GSX_REQUIRE(((uintptr_t)qvec & 15) == 0 && ((uintptr_t)grad_qvec & 15) == 0 &&
                  ((uintptr_t)grad_cov2d & 15) == 0 && ((uintptr_t)grad_mean2d & 7) == 0,
              "qvec, grad_qvec, grad_cov2d must be 16-byte aligned, grad_mean2d 8-byte");
  return launch_project_backward(n, mean, qvec, log_scale, alpha_logit, *cam, counts,
                                 grad_mean2d, grad_cov2d, grad_alpha, grad_mean, grad_qvec,
                                 grad_log_scale, grad_alpha_logit, grad_flags, as_stream(stream));
}


// ---------------------------------------------------------------- densify
int gsx_densify_count_visible(int64_t n, const int32_t *counts, int32_t *cnt, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(n >= 0, "n must be >= 0");
  GSX_REQUIRE(n == 0 || (counts && cnt), "null pointer argument");
  return launch_count_visible(n, counts, cnt, as_stream(stream));
}

int gsx_densify_accumulate(int64_t n, const float *grad, int32_t dim, const int32_t *counts,
                           float *grad_accum, int32_t reduce_max, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(n >= 0, "n must be >= 0");
  GSX_REQUIRE(dim == 2 || dim == 3, "dim must be 2 or 3 (got %d)", dim);
  GSX_REQUIRE(n == 0 || (grad && grad_accum), "null pointer argument");
  return launch_accumulate_norm(n, grad, dim, counts, grad_accum, reduce_max ? 1 : 0,
                                as_stream(stream));
}

int gsx_densify_classify(int64_t n, const float *grad_accum, const int32_t *cnt,
                         const float *log_scale, float grad_thresh, float scale_thresh,
                         int32_t divide_by_count, uint8_t *cls, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(n >= 0, "n must be >= 0");
  GSX_REQUIRE(n == 0 || (grad_accum && log_scale && cls && (cnt || !divide_by_count)),
              "null pointer argument");
  return launch_classify(n, grad_accum, cnt, log_scale, grad_thresh, scale_thresh,
                         divide_by_count ? 1 : 0, cls, as_stream(stream));
}

int gsx_densify_rewrite(int64_t n, const uint8_t *cls, const int64_t *pos_stay,
                        const int64_t *pos_clone, const int64_t *pos_split, int64_t n_stay,
                        int64_t n_clone, int64_t n_split, const float *mean, const float *qvec,
                        const float *log_scale, const float *sh, int32_t sh_len,
                        const float *alpha_logit, float shrink, uint64_t seed, float *out_mean,
                        float *out_qvec, float *out_log_scale, float *out_sh, float *out_alpha_logit,
                        void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(n >= 0 && n_stay >= 0 && n_clone >= 0 && n_split >= 0, "negative size");
  GSX_REQUIRE(n_stay + n_split == n, "every Gaussian either stays or is split");
  GSX_REQUIRE(sh_len > 0, "sh_len must be positive");
  GSX_REQUIRE(shrink > 0.0f, "shrink factor must be positive");
  GSX_REQUIRE(n == 0 || (cls && pos_stay && pos_clone && pos_split && mean && qvec && log_scale &&
                         sh && alpha_logit && out_mean && out_qvec && out_log_scale && out_sh &&
                         out_alpha_logit),
              "null pointer argument");
  return launch_rewrite(n, cls, pos_stay, pos_clone, pos_split, n_stay, n_clone, n_split, mean,
                        qvec, log_scale, sh, sh_len, alpha_logit, logf(shrink), seed, out_mean,
                        out_qvec, out_log_scale, out_sh, out_alpha_logit, as_stream(stream));
}


// ---------------------------------------------------------------- training
size_t gsx_adam_group_size(void) { return sizeof(gsx_adam_group); }

size_t gsx_photometric_loss_workspace_bytes(int32_t height, int32_t width) {
  if (height <= 0 || width <= 0) return 0;
  return loss_workspace_bytes(height, width);
}

int64_t gsx_photometric_loss_blocks(int32_t height, int32_t width) {
  if (height <= 0 || width <= 0) return 0;
  return (3 * (int64_t)height * width + 255) / 256;
}

int gsx_photometric_loss(const float *out, const float *gt, int32_t height, int32_t width,
                         int32_t win_size, float ssim_mult, int32_t l2, float *grad_out,
                         float *partials, void *workspace, size_t workspace_bytes, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(height > 0 && width > 0, "image size must be positive");
  GSX_REQUIRE(win_size >= 1 && win_size <= 31 && (win_size & 1),
              "win_size must be odd, 1..31 (got %d; kornia centres an even window between "
              "pixels, which these kernels do not)",
              win_size);
  GSX_REQUIRE(win_size / 2 < height && win_size / 2 < width,
              "reflected borders need the window radius below the image size");
  GSX_REQUIRE(ssim_mult >= 0.0f && ssim_mult <= 1.0f, "ssim_mult must be in [0, 1]");
  GSX_REQUIRE(out && gt && grad_out && workspace, "null pointer argument");
  GSX_REQUIRE(workspace_bytes >= loss_workspace_bytes(height, width),
              "loss workspace too small: %zu < %zu bytes", workspace_bytes,
              loss_workspace_bytes(height, width));
  return run_ssim_loss(out, gt, height, width, win_size, ssim_mult, l2 ? 1 : 0, grad_out, partials,
                       workspace, as_stream(stream));
}

int gsx_adam_step(const gsx_adam_group *groups_dev, const int64_t *offsets_dev, int32_t n_groups,
                  int64_t total, void *stream) {
  g_err[0] = 0;
  GSX_REQUIRE(n_groups >= 1 && total >= 0, "need at least one group and total >= 0");
  GSX_REQUIRE(groups_dev && offsets_dev, "null pointer argument");
  return launch_adam(groups_dev, n_groups, total, offsets_dev, as_stream(stream));
}

}  // extern "C"
