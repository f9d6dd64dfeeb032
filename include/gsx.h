/*
 * gsx.h -- C ABI of the GB300 (sm_103a) Gaussian-splatting rasteriser.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (cudaStream_t passed as void*; NULL = legacy default stream) and returns an
 * int status (GSX_OK = 0).  No entry point exits the process, traps on the
 * device or allocates device memory: scratch space is passed in by the caller
 * (size from the matching *_workspace_bytes query).  Unless stated otherwise a
 * call only enqueues work on `stream` and returns without synchronising.
 *
 * Two groups of entry points:
 *  1. the four hot-path functions of the reference's pybind module `_gs`
 *     (gs/src/bindings.cpp:6-7, 29, 42-48), with the same argument order and
 *     meaning and the same in-place output convention;
 *  2. the fused native path used by gaussian_splatting_3d_gb300's renderer:
 *     projection (cull + EWA + AABB count), deterministic tile binning,
 *     the raster forward and backward with a per-channel SH stride, and the
 *     projection backward.
 */
#ifndef GSX_H
#define GSX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  GSX_OK = 0,
  GSX_ERR_INVALID_ARG = 1, /* bad size, null pointer, unsupported option */
  GSX_ERR_CAPACITY = 2,    /* caller-provided buffer or workspace too small */
  GSX_ERR_TIMEOUT = 3,     /* a bounded device-side wait gave up */
  GSX_ERR_CUDA = 4,        /* a CUDA runtime call failed */
  GSX_ERR_MISMATCH = 5     /* inputs disagree with a caller-stated size */
};

/* Human-readable name of a status code. */
const char *gsx_status_string(int status);
/* Detail message of the last failing call on this host thread ("" if none). */
const char *gsx_last_error(void);
/* ABI version of this library (increments on any signature change). */
/* 2: gsx_project_backward / gsx_batch_project_backward take grad_flags;
   3: gsx_raster_params gains pixels_per_thread, gsx_batch_view's spare
      int32 becomes pixels_per_thread, the batched raster passes take
      tile_order and work_counter */
#define GSX_ABI_VERSION 3
int gsx_abi_version(void);
/* Number of kernels this library has launched in this process so far. */
uint64_t gsx_kernel_launch_count(void);

/* ---- 1. reference `_gs` hot-path entry points --------------------------- */

/*
 * Replaces `culling_gaussian_bsphere` (gs/src/render.cu:15-43; kernel
 * gs/src/include/culling.h:11-20).  mask[i] = 1 iff the sphere at mean[i]
 * with radius max(svec[i]) * thresh is on or in front of all six planes
 * (normal[6,3], pts[6,3]).  qvec is accepted and unused, as in the reference.
 */
int gsx_culling_gaussian_bsphere(int64_t n, const float *mean, const float *qvec,
                                 const float *svec, const float *normal,
                                 const float *pts, uint8_t *mask, float thresh,
                                 void *stream);

/*
 * Workspace for gsx_tile_culling_aabb_start_end and gsx_bin_gaussians:
 * n_gaussians Gaussians, up to key_capacity (tile, Gaussian) keys, n_tiles tiles.
 * The workspace must start on a 256-byte boundary (as cudaMalloc returns);
 * the binning calls reject others with GSX_ERR_INVALID_ARG.
 */
size_t gsx_binning_workspace_bytes(int64_t n_gaussians, int64_t key_capacity,
                                   int64_t n_tiles);

/*
 * Replaces `tile_culling_aabb_start_end` (gs/src/render.cu:380-397;
 * gs/src/include/aabb_culling.h:192-260).  aabb_topleft / aabb_bottomright
 * are int32 [n,2] tile rectangles (inclusive), depth float [n].  Writes
 * gaussian_ids[n_keys] sorted by (tile, depth bits) with equal keys in index
 * order, and start/end[n_tiles_h*n_tiles_w] (-1 for tiles without keys).
 * Like the reference it synchronises `stream` once, to check that the
 * rectangles hold exactly n_keys keys (GSX_ERR_MISMATCH otherwise).
 */
int gsx_tile_culling_aabb_start_end(int64_t n, int64_t n_keys,
                                    const int32_t *aabb_topleft,
                                    const int32_t *aabb_bottomright,
                                    const float *depth, int32_t n_tiles_h,
                                    int32_t n_tiles_w, int32_t *gaussian_ids,
                                    int32_t *start, int32_t *end, void *workspace,
                                    size_t workspace_bytes, void *stream);

/*
 * Same binning as gsx_tile_culling_aabb_start_end, for callers that cannot
 * allocate device memory: a plugin inside another application's fixed
 * memory budget, or a real-time loop that must never enter the allocator
 * (cudaMalloc can synchronise the device).  It takes no workspace and
 * allocates nothing; its scratch is a 64 MiB array in the library's static
 * device memory, which every GPU that loads the library holds until the
 * process exits.  Inputs are accepted when
 * gsx_binning_workspace_bytes(n, n_keys, n_tiles_h * n_tiles_w) <= 64 MiB
 * (about 17.0 bytes per Gaussian plus 17.4 bytes per key: some 1.9 million
 * Gaussians with as many keys) and rejected with GSX_ERR_CAPACITY otherwise.
 * The first call in each CUDA context (the device's primary context, or a
 * context the caller made current) looks up the array's device address in
 * that context; make that first call before any stream capture.  Like
 * gsx_tile_culling_aabb_start_end it synchronises `stream` once.  All calls
 * share the array, so calls that overlap on the GPU (other streams, other
 * host threads) race and must be serialised by the caller.  This entry point
 * has no counterpart in the reference.
 */
int gsx_tile_culling_aabb_start_end_noalloc(int64_t n, int64_t n_keys,
                                            const int32_t *aabb_topleft,
                                            const int32_t *aabb_bottomright,
                                            const float *depth, int32_t n_tiles_h,
                                            int32_t n_tiles_w, int32_t *gaussian_ids,
                                            int32_t *start, int32_t *end, void *stream);

/*
 * Replaces `tile_based_vol_rendering_sh` (gs/src/render.cu:483-544; kernel
 * gs/src/include/vol_render_sh.h:171-248).  mean f32[n,2], cov f32[n,2,2],
 * sh_coeffs f32[n,3,C*C], alpha f32[n], start/end i32[n_tiles],
 * gaussian_ids i32[n_keys], out f32[H*W*3] (pre-zeroed; pixels of empty
 * tiles are left untouched), topleft f32[2] and c2w f32[3,4] in device
 * memory.  C (SH order = degree + 1) in 1..4; tile_size*tile_size <= 1024.
 */
int gsx_tile_based_vol_rendering_sh(
    int64_t n, int64_t n_keys, const float *mean, const float *cov,
    const float *sh_coeffs, const float *alpha, const int32_t *start,
    const int32_t *end, const int32_t *gaussian_ids, float *out,
    const float *topleft, const float *c2w, uint32_t tile_size,
    uint32_t n_tiles_h, uint32_t n_tiles_w, float pixel_size_x,
    float pixel_size_y, uint32_t H, uint32_t W, uint32_t C, float thresh,
    void *stream);

/*
 * Replaces `tile_based_vol_rendering_backward_sh` (gs/src/render.cu:546-624;
 * kernel gs/src/include/vol_render_sh.h:353-455).  Same inputs as the
 * forward plus out (the forward image) and grad_out f32[H*W*3]; adds into
 * grad_mean f32[n,2], grad_cov f32[n,2,2] (slots 1 and 2 receive the same
 * value), grad_sh_coeffs f32[n,3,C*C], grad_alpha f32[n] (pre-zeroed).
 */
int gsx_tile_based_vol_rendering_backward_sh(
    int64_t n, int64_t n_keys, const float *mean, const float *cov,
    const float *sh_coeffs, const float *alpha, const int32_t *start,
    const int32_t *end, const int32_t *gaussian_ids, const float *out,
    float *grad_mean, float *grad_cov, float *grad_sh_coeffs, float *grad_alpha,
    const float *grad_out, const float *topleft, const float *c2w,
    uint32_t tile_size, uint32_t n_tiles_h, uint32_t n_tiles_w,
    float pixel_size_x, float pixel_size_y, uint32_t H, uint32_t W, uint32_t C,
    float thresh, void *stream);

/* ---- 2. fused native path ---------------------------------------------- */

/* Pinhole camera; c2w is the [3,4] row-major camera-to-world matrix used by
 * the reference (utils/camera.py:219-303); frustum planes as get_frustum
 * returns them (normals normalised).  */
typedef struct gsx_camera {
  float c2w[12];
  float fx, fy, cx, cy;
  int32_t width, height;
  float frustum_normals[18]; /* [6,3] */
  float frustum_pts[18];     /* [6,3] */
} gsx_camera;

/*
 * One view of a batched pass.  The views of a batch are described by an
 * array of these in device memory (plus the same array on the host for sizes).
 * Each view names its scene (which may be shared with other views), its
 * camera and image, where its (view, Gaussian) items start in the per-item
 * arrays and where its tiles start in the global tile numbering.
 */
typedef struct gsx_batch_view {
  const float *mean, *qvec, *log_scale, *alpha_logit, *sh; /* the view's scene */
  float *g_mean, *g_qvec, *g_log_scale, *g_alpha_logit;    /* scene gradients (backward) */
  float *g_sh;                                             /* SH gradient [n,3,sh_stride] */
  int64_t n_gaussians;  /* Gaussians in the scene */
  int64_t item_offset;  /* first item of this view: items are (view, Gaussian) pairs */
  int64_t tile_offset;  /* first global tile of this view */
  int32_t sh_stride, sh_order;
  int32_t tile_w, tile_h, n_tiles_w, n_tiles_h;
  float topleft[2];
  float pixel_size_x, pixel_size_y;
  float *out;            /* [height, width, 3] */
  const float *grad_out; /* dL/dout [height, width, 3] (backward) */
  int32_t write_empty_tiles;
  int32_t pixels_per_thread; /* raster schedule as in gsx_raster_params; the same in every view */
  gsx_camera cam;
} gsx_batch_view;

/* sizeof(gsx_batch_view), for bindings that build the table themselves. */
size_t gsx_batch_view_size(void);

/*
 * Batched passes over n_views views (table in device memory, views_dev, and
 * the same table on the host, views_host).  Per-item arrays (mean2d f32[I,2],
 * cov2d f32[I,4], depth f32[I], alpha f32[I], rect i32[I,4], counts i32[I],
 * g_mean2d, g_cov2d, g_alpha) have I = sum of the views' n_gaussians entries;
 * start/end have one entry per tile of the batch (sum of the views' tiles).
 * All views share the tile shape and the SH order.  The binning is
 * asynchronous (read its key count with gsx_binning_status using I as the
 * Gaussian count).  gsx_batch_project_backward needs all views to share one
 * scene and writes that scene's gradients (views[0].g_*), summed over views
 * (grad_flags as for gsx_project_backward); the raster backward adds SH
 * gradients into each view's g_sh.
 */
int gsx_batch_project_forward(const gsx_batch_view *views_dev, const gsx_batch_view *views_host,
                              int32_t n_views, float frustum_radius, float tile_radius,
                              float *mean2d, float *cov2d, float *depth, float *alpha,
                              int32_t *rect, int32_t *counts, void *stream);
int gsx_batch_bin_async(const gsx_batch_view *views_dev, const gsx_batch_view *views_host,
                        int32_t n_views, const int32_t *rect, const int32_t *counts,
                        const float *depth, int64_t key_capacity, int32_t *gaussian_ids,
                        int32_t *start, int32_t *end, void *workspace, size_t workspace_bytes,
                        void *stream);
/*
 * The batched raster passes.  tile_order (i32[total tiles], e.g. from
 * gsx_tile_order over the batch's start/end; NULL = tile index order) and
 * work_counter (one u32 of device memory; NULL = one CTA per tile) make the
 * launch persistent: as many CTAs as the SMs hold at once claim the tiles,
 * longest lists first, one atomic per tile.  The counter is zeroed on
 * `stream` before the launch; the two passes may share it when they run on
 * one stream.  Images and gradients do not depend on either.
 */
int gsx_batch_render_forward(const gsx_batch_view *views_dev, const gsx_batch_view *views_host,
                             int32_t n_views, int64_t key_capacity, const float *mean2d,
                             const float *cov2d, const float *alpha, const int32_t *start,
                             const int32_t *end, const int32_t *gaussian_ids, float T_thresh,
                             const int32_t *tile_order, uint32_t *work_counter, void *stream);
int gsx_batch_render_backward(const gsx_batch_view *views_dev, const gsx_batch_view *views_host,
                              int32_t n_views, int64_t key_capacity, const float *mean2d,
                              const float *cov2d, const float *alpha, const int32_t *start,
                              const int32_t *end, const int32_t *gaussian_ids, float *g_mean2d,
                              float *g_cov2d, float *g_alpha, float T_thresh,
                              const int32_t *tile_order, uint32_t *work_counter, void *stream);
int gsx_batch_project_backward(const gsx_batch_view *views_dev, const gsx_batch_view *views_host,
                               int32_t n_views, const int32_t *counts, const float *g_mean2d,
                               const float *g_cov2d, const float *g_alpha, int32_t grad_flags,
                               void *stream);

/*
 * One pass over n Gaussians (mean f32[n,3], qvec f32[n,4] WXYZ,
 * log_scale f32[n,3], alpha_logit f32[n]): scale = exp(log_scale),
 * alpha = sigmoid(alpha_logit), bounding-sphere cull (radius factor
 * frustum_radius), projection to normalised image coordinates with depth
 * and J treated as the reference treats them (gs/renderer.py:365-419),
 * the AABB tile rectangle (gs/culling.py:8-37 with tile_radius = D) and its
 * key count.  Outputs: mean2d f32[n,2], cov2d f32[n,4], depth f32[n],
 * alpha f32[n], rect i32[n,4] (tlx, tly, brx, bry), counts i32[n]
 * (0 = culled).  If scales_are_activated != 0, log_scale holds exp(.) already.
 */
int gsx_project_forward(int64_t n, const float *mean, const float *qvec,
                        const float *log_scale, const float *alpha_logit,
                        const gsx_camera *cam, float frustum_radius,
                        float tile_radius, int32_t tile_w, int32_t tile_h,
                        int32_t scales_are_activated, float *mean2d, float *cov2d,
                        float *depth, float *alpha, int32_t *rect,
                        int32_t *counts, void *stream);

/*
 * Deterministic tile binning of n Gaussians from their rectangles
 * (rect i32[n,4]), counts and depth: sort by depth bits, exclusive scan of
 * counts in that order, key emission, stable sort by tile.  Results equal the
 * reference's stable 64-bit sort of (tile << 32 | depth bits) keys with equal
 * keys in index order.  Writes gaussian_ids[<= key_capacity], start/end
 * (n_tiles_w*n_tiles_h, -1 = empty) and, on the host, *n_keys_out.
 * Synchronises `stream` once to read the key count.  If the count exceeds
 * key_capacity nothing past the count is written and GSX_ERR_CAPACITY is
 * returned with *n_keys_out set, so the caller can grow and call again.
 */
int gsx_bin_gaussians(int64_t n, const int32_t *rect, const int32_t *counts,
                      const float *depth, int32_t n_tiles_w, int32_t n_tiles_h,
                      int64_t key_capacity, int32_t *gaussian_ids, int32_t *start,
                      int32_t *end, int64_t *n_keys_out, void *workspace,
                      size_t workspace_bytes, void *stream);

/*
 * The same binning without any host synchronisation (capturable in a CUDA
 * graph): keys beyond key_capacity are not written, and the key total and
 * error bits stay in the workspace.  gsx_binning_status reads them later
 * (synchronising `stream`) and returns GSX_ERR_CAPACITY if the capacity was
 * too small, in which case the lists are incomplete.
 */
int gsx_bin_gaussians_async(int64_t n, const int32_t *rect, const int32_t *counts,
                            const float *depth, int32_t n_tiles_w, int32_t n_tiles_h,
                            int64_t key_capacity, int32_t *gaussian_ids, int32_t *start,
                            int32_t *end, void *workspace, size_t workspace_bytes,
                            void *stream);
/*
 * Diagnostic of the sort's bounded look-back wait (no reference counterpart):
 * a single CTA claims chunk 1 of a two-chunk pass and waits for chunk 0,
 * which never publishes; the wait gives up after its poll limit and sets the
 * timeout bit.  Returns GSX_ERR_TIMEOUT when the path works (error_bits, if
 * not NULL, receives the raw bits).  Synchronises `stream`; scratch is
 * caller device memory of gsx_look_back_selftest_bytes(), 256-byte aligned.
 */
size_t gsx_look_back_selftest_bytes(void);
int gsx_look_back_selftest(void *scratch, size_t scratch_bytes, uint32_t *error_bits, void *stream);

int gsx_binning_status(const void *workspace, int64_t n_gaussians, int64_t key_capacity,
                       int32_t n_tiles_w, int32_t n_tiles_h, int64_t *n_keys_out,
                       void *stream);

/*
 * Non-blocking form of gsx_binning_status, for callers that keep several
 * binnings in flight (no reference counterpart: the reference's binning
 * always synchronises).  gsx_binning_status_copy_async enqueues on `stream`
 * a copy of the binning's 16-byte status block (u64 key total, u32 error
 * bits, u32 key count used) into dst (pinned host or device memory);
 * gsx_binning_status_decode turns a block that has arrived into the status
 * gsx_binning_status would return, and the key total.
 */
int gsx_binning_status_copy_async(const void *workspace, int64_t n_gaussians,
                                  int64_t key_capacity, void *dst, void *stream);
int gsx_binning_status_decode(const void *block, int64_t key_capacity, int32_t n_tiles_w,
                              int32_t n_tiles_h, int64_t *n_keys_out);

/* Raster parameters of the fused path. */
typedef struct gsx_raster_params {
  int32_t width, height;
  int32_t tile_w, tile_h;       /* tile_w*tile_h threads per tile, <= 1024 */
  int32_t n_tiles_w, n_tiles_h;
  int32_t sh_order;             /* C = SH degree + 1, 1..4 */
  int32_t sh_stride;            /* floats per colour channel in sh (>= C*C) */
  float pixel_size_x, pixel_size_y;
  float T_thresh;
  int32_t write_empty_tiles;    /* 1: write zeros for pixels of empty tiles */
  int32_t pixels_per_thread;    /* raster schedule: pixels per thread, 1 or 2
                                   (2 needs tile_w and tile_h multiples of 8,
                                   else 1 is used; the forward with a
                                   background or maps always uses 1); 0 = the
                                   faster measured choice: 1 for the forward,
                                   2 for the backward.  Images are identical,
                                   gradients agree within rounding. */
} gsx_raster_params;

/* Forward raster over precomputed per-Gaussian mean2d/cov2d/alpha, SH
 * coefficients sh f32[n,3,sh_stride]; topleft f32[2] and c2w f32[3,4] in
 * device memory. */
int gsx_render_forward(const gsx_raster_params *p, int64_t n, int64_t n_keys,
                       const float *mean2d, const float *cov2d, const float *sh,
                       const float *alpha, const int32_t *start, const int32_t *end,
                       const int32_t *gaussian_ids, const float *topleft,
                       const float *c2w, float *out, void *stream);

/*
 * gsx_render_forward with a background and output maps (no reference
 * counterpart: the reference's background variant, vol_render_bg.h, does not
 * compile).  bg_rgb (host pointer to 3 floats, or NULL): out += T_final * bg,
 * where T_final is the transmittance left when the pixel stops; passing that
 * image to gsx_render_backward makes the gradients exact for it.
 * alpha_out f32[H*W] (or NULL) = 1 - T_final; depth_out f32[H*W] (or NULL) =
 * sum over the composited Gaussians of T a G z with z = depth[i] (the
 * projection's camera depth, f32[n]).  Empty tiles give bg, 0, 0.
 */
int gsx_render_forward_maps(const gsx_raster_params *params, int64_t n, int64_t n_keys,
                            const float *mean2d, const float *cov2d, const float *sh,
                            const float *alpha, const int32_t *start, const int32_t *end,
                            const int32_t *gaussian_ids, const float *topleft, const float *c2w,
                            float *out, const float *bg_rgb, const float *depth,
                            float *alpha_out, float *depth_out, void *stream);

/*
 * Scheduling order for the forward raster (no reference counterpart):
 * tile_order i32[n_tiles] receives the tiles sorted by descending list length
 * end - start, in log-spaced classes (8 per doubling; the order inside a
 * class is unspecified).  Longest lists first shortens the tail of the grid.
 */
int gsx_tile_order(const int32_t *start, const int32_t *end, int32_t n_tiles, int32_t *tile_order,
                   void *stream);

/* gsx_render_forward with CTA b rendering tile tile_order[b]; tile_order must
 * be a permutation of the n_tiles_w * n_tiles_h tiles (entries outside the
 * grid render nothing).  The image does not depend on the order. */
int gsx_render_forward_ordered(const gsx_raster_params *p, int64_t n, int64_t n_keys,
                               const float *mean2d, const float *cov2d, const float *sh,
                               const float *alpha, const int32_t *start, const int32_t *end,
                               const int32_t *gaussian_ids, const float *topleft,
                               const float *c2w, float *out, const int32_t *tile_order,
                               void *stream);

/*
 * Opt-in per-Gaussian colours (no reference counterpart: the reference
 * evaluates SH per pixel, gs/src/include/vol_render_sh.h:139-141, 208-217).
 * gsx_project_colors writes rgb f32[n,3] = sigmoid(sh . Y(dir)) with dir the
 * unit vector from cam_pos (host float[3], the camera centre) to mean[i], the
 * reference's SH basis and sigmoid colour; Gaussians with counts[i] <= 0
 * (counts may be NULL) get 0.  gsx_project_colors_backward overwrites
 * grad_sh f32[n,3,sh_stride] from grad_rgb f32[n,3] and ADDS the gradient
 * through the direction into grad_mean f32[n,3] (so it runs after
 * gsx_project_backward).  gsx_render_forward_rgb / gsx_render_backward_rgb
 * composite those colours (no per-pixel SH; grad_rgb is added into, the caller
 * zeroes it); tile_order may be NULL or as for the *_ordered entry points.
 */
int gsx_project_colors(int64_t n, const float *mean, const float *sh, int32_t sh_stride,
                       int32_t sh_order, const float *cam_pos, const int32_t *counts, float *rgb,
                       void *stream);
int gsx_project_colors_backward(int64_t n, const float *mean, const float *sh, int32_t sh_stride,
                                int32_t sh_order, const float *cam_pos, const int32_t *counts,
                                const float *rgb, const float *grad_rgb, float *grad_sh,
                                float *grad_mean, void *stream);
int gsx_render_forward_rgb(const gsx_raster_params *p, int64_t n, int64_t n_keys,
                           const float *mean2d, const float *cov2d, const float *rgb,
                           const float *alpha, const int32_t *start, const int32_t *end,
                           const int32_t *gaussian_ids, const float *topleft, const float *c2w,
                           float *out, const int32_t *tile_order, void *stream);
int gsx_render_backward_rgb(const gsx_raster_params *p, int64_t n, int64_t n_keys,
                            const float *mean2d, const float *cov2d, const float *rgb,
                            const float *alpha, const int32_t *start, const int32_t *end,
                            const int32_t *gaussian_ids, const float *topleft, const float *c2w,
                            const float *out, const float *grad_out, float *grad_mean2d,
                            float *grad_cov2d, float *grad_rgb, float *grad_alpha,
                            const int32_t *tile_order, void *stream);

/* Backward raster; grad_* are added into (caller zeroes them). */
int gsx_render_backward(const gsx_raster_params *p, int64_t n, int64_t n_keys,
                        const float *mean2d, const float *cov2d, const float *sh,
                        const float *alpha, const int32_t *start,
                        const int32_t *end, const int32_t *gaussian_ids,
                        const float *topleft, const float *c2w, const float *out,
                        const float *grad_out, float *grad_mean2d,
                        float *grad_cov2d, float *grad_sh, float *grad_alpha,
                        void *stream);

/*
 * Sticky error bits of every raster launch of this process on the current
 * device (no reference counterpart: the reference's kernels trap instead).
 * Bit 0: a wait for the bulk copies (cp.async.bulk) that stage a batch's SH
 * rows in shared memory gave up; that tile's output or gradients are
 * incomplete.  Synchronises `stream`; clear != 0 resets the bits.
 */
int gsx_raster_status(uint32_t *flags, int32_t clear, void *stream);

/*
 * Diagnostic of the failure path above (no reference counterpart): one CTA
 * polls a barrier phase that cannot complete, gives up after `limit` polls
 * (1 <= limit <= 2^20), sets bit 0 of the raster status and writes the polls
 * made to polls_dev[0] (device memory).  Nothing faults or hangs; the context
 * stays usable.
 */
int gsx_raster_wait_selftest(uint32_t limit, uint32_t *polls_dev, void *stream);

/*
 * Diagnostic of the raster's exponential (no reference counterpart; the
 * reference calls CUDA's expf at gs/src/include/kernels.h:188): out[i] for
 * x[i], i < n, both device memory, through the scalar form used by the
 * projection and the CPU oracle (variant 0), the branch-free form for
 * exponents <= 0 of the raster kernels (1), or its paired float2 form on
 * (x[2k], x[2k+1]) (2).  Enqueued on `stream`.
 */
int gsx_exp_selftest(const float *x, int64_t n, float *out, int32_t variant, void *stream);

/* gsx_render_backward with CTA b working on tile tile_order[b] (the same
 * contract as gsx_render_forward_ordered; the gradients do not depend on the
 * order beyond the summation order of their float additions). */
int gsx_render_backward_ordered(const gsx_raster_params *p, int64_t n, int64_t n_keys,
                                const float *mean2d, const float *cov2d, const float *sh,
                                const float *alpha, const int32_t *start, const int32_t *end,
                                const int32_t *gaussian_ids, const float *topleft,
                                const float *c2w, const float *out, const float *grad_out,
                                float *grad_mean2d, float *grad_cov2d, float *grad_sh,
                                float *grad_alpha, const int32_t *tile_order, void *stream);

/*
 * Projection backward from the raster gradients grad_mean2d f32[n,2],
 * grad_cov2d f32[n,4], grad_alpha f32[n] to the parameter gradients
 * grad_mean f32[n,3], grad_qvec f32[n,4], grad_log_scale f32[n,3],
 * grad_alpha_logit f32[n] (overwritten; zero for culled Gaussians, i.e.
 * counts[i] == 0).  grad_flags = 0 gives the reference's gradient
 * (gs/renderer.py:365-419: depth detached in mean2d = p_xy / p_z, J built
 * without gradient; vol_render_sh.h:346: the opacity clamp min(alpha, 0.99)
 * ignored).  GSX_GRAD_DEPTH adds the z term of mean2d (the reference's
 * depth_detach=False), GSX_GRAD_JACOBIAN the gradient through J,
 * GSX_GRAD_CLAMP zeroes the opacity gradient where the clamp is active;
 * GSX_GRAD_EXACT (all three) is the true derivative of the rendered image.
 */
#define GSX_GRAD_DEPTH 1
#define GSX_GRAD_JACOBIAN 2
#define GSX_GRAD_CLAMP 4
#define GSX_GRAD_EXACT 7
int gsx_project_backward(int64_t n, const float *mean, const float *qvec,
                         const float *log_scale, const float *alpha_logit,
                         const gsx_camera *cam, const int32_t *counts,
                         const float *grad_mean2d, const float *grad_cov2d,
                         const float *grad_alpha, float *grad_mean,
                         float *grad_qvec, float *grad_log_scale,
                         float *grad_alpha_logit, int32_t grad_flags, void *stream);


/*
 * Adaptive density control (no reference counterpart at this boundary: the
 * reference does these steps with torch ops in gs/sh_renderer.py:216,
 * 426-540, 602-623).
 *   gsx_densify_count_visible: cnt[i] += 1 where counts[i] > 0 (i.e. Gaussian
 *     i survived frustum culling in the last projection).
 *   gsx_densify_accumulate: grad_accum[i] = max(grad_accum[i], |grad[i]|)
 *     (reduce_max) or += |grad[i]|, grad f32[n,dim] (dim 3: dL/dmean, dim 2:
 *     dL/dmean2d); with counts, only where counts[i] > 0.
 *   gsx_densify_classify: cls[i] = 0 keep, 1 clone, 2 split: the statistic
 *     (divided by cnt + 1e-5 when divide_by_count) above grad_thresh, split
 *     when any exp(log_scale) > scale_thresh.
 *   gsx_densify_rewrite: the new arrays [not split, in order] ++ [clones] ++
 *     [split samples: copy 0 of every split Gaussian, then copy 1], from the
 *     exclusive prefix counts of (cls != 2), (cls == 1), (cls == 2); a split
 *     sample is mean + R(q)^T (n * scale), n ~ N(0,1) from a counter-based
 *     generator keyed by seed, with log-scale log(scale / shrink).
 */
int gsx_densify_count_visible(int64_t n, const int32_t *counts, int32_t *cnt, void *stream);
int gsx_densify_accumulate(int64_t n, const float *grad, int32_t dim, const int32_t *counts,
                           float *grad_accum, int32_t reduce_max, void *stream);
int gsx_densify_classify(int64_t n, const float *grad_accum, const int32_t *cnt,
                         const float *log_scale, float grad_thresh, float scale_thresh,
                         int32_t divide_by_count, uint8_t *cls, void *stream);
int gsx_densify_rewrite(int64_t n, const uint8_t *cls, const int64_t *pos_stay,
                        const int64_t *pos_clone, const int64_t *pos_split, int64_t n_stay,
                        int64_t n_clone, int64_t n_split, const float *mean, const float *qvec,
                        const float *log_scale, const float *sh, int32_t sh_len,
                        const float *alpha_logit, float shrink, uint64_t seed, float *out_mean,
                        float *out_qvec, float *out_log_scale, float *out_sh, float *out_alpha_logit,
                        void *stream);


/*
 * Training-step kernels (utils/loss.py:5-24, gs/sh_renderer.py:720-729).
 *
 * gsx_photometric_loss: for HWC float32 images out, gt [H,W,3] writes
 * grad_out = dL/dout of L = ssim_mult * mean(clamp((1 - SSIM)/2, 0, 1)) +
 * (1 - ssim_mult) * (l2 ? mean((out-gt)^2) : mean|out-gt|), SSIM with an
 * odd win_size (<= 31) Gaussian window of sigma 1.5, reflected borders,
 * C1 = 1e-4, C2 = 9e-4, eps 1e-12 (kornia's published definition).  The loss
 * value is sum(partials[0:nb]) * ssim_mult / (3HW) + sum(partials[nb:2nb]) *
 * (1 - ssim_mult) / (3HW), nb = gsx_photometric_loss_blocks(H, W) (partials:
 * 2*nb floats of device memory; may be NULL).
 *
 * gsx_adam_step: one torch.optim.Adam step over every group of a device
 * table: m += (1-b1)(g-m); v = b2 v + (1-b2) g^2;
 * p -= step_size * m / (sqrt(v) / bias_correction2_sqrt + eps), where the
 * caller sets step_size = lr / (1 - b1^t), bias_correction2_sqrt =
 * sqrt(1 - b2^t).  offsets_dev[i] = first element of group i in the
 * concatenation (offsets_dev[0] = 0), total = all elements.
 */
typedef struct gsx_adam_group {
  float *param;
  const float *grad;
  float *exp_avg;
  float *exp_avg_sq;
  int64_t n;
  float step_size;
  float bias_correction2_sqrt;
  float beta1, beta2, eps;
  int32_t reserved;
} gsx_adam_group;

size_t gsx_adam_group_size(void);
size_t gsx_photometric_loss_workspace_bytes(int32_t height, int32_t width);
int64_t gsx_photometric_loss_blocks(int32_t height, int32_t width);
int gsx_photometric_loss(const float *out, const float *gt, int32_t height, int32_t width,
                         int32_t win_size, float ssim_mult, int32_t l2, float *grad_out,
                         float *partials, void *workspace, size_t workspace_bytes, void *stream);
int gsx_adam_step(const gsx_adam_group *groups_dev, const int64_t *offsets_dev, int32_t n_groups,
                  int64_t total, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GSX_H */
