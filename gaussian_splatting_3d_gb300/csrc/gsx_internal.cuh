// gsx_internal.cuh -- device helpers shared by the sm_103a kernels.
//
// Arithmetic contract (every kernel is compiled with -fmad=false, so only the
// fmaf() calls written here fuse; division and sqrtf are IEEE round-to-nearest,
// denormals are kept):
//   * gsx_expf: Cody-Waite reduction with a two-part ln2 (the float split
//     0.693145751953125 + 1.428606765330187045e-06 that the SLEEF library
//     publishes), degree-7 Taylor polynomial, 2^j through the exponent bits,
//     +0 below -87.  The same
//     operation sequence is restated in the CPU oracle, so the two agree bit
//     for bit; it replaces the CUDA expf calls of the reference
//     (gs/src/include/kernels.h:188, shencoder.h:4).
//   * fmaf() sits where nvcc contracts the reference's a*b+c expressions.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gsx.h"

namespace gsx {

constexpr float kMinRenderAlpha = 1.0f / 255.0f;  // gs/src/include/common.h:89

__device__ __forceinline__ float gsx_expf(float x) {
  if (!(x > -87.0f)) return (x != x) ? x : 0.0f;
  if (x > 88.75f) return __int_as_float(0x7f800000);
  float t = fmaf(x, 1.44269502162933349609375f, 12582912.0f);
  float j = t - 12582912.0f;
  float r = fmaf(j, -0.693145751953125f, x);
  r = fmaf(j, -1.428606765330187045e-06f, r);
  float p = 1.98412698412698412e-04f;
  p = fmaf(p, r, 1.38888888888888889e-03f);
  p = fmaf(p, r, 8.33333333333333333e-03f);
  p = fmaf(p, r, 4.16666666666666667e-02f);
  p = fmaf(p, r, 1.66666666666666667e-01f);
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  int ji = (int)j;
  if (ji > 127) {
    p = p * 2.0f;
    ji -= 1;
  }
  return p * __int_as_float((ji + 127) << 23);
}

// gsx_expf for x in (-87, 0]: the same operation sequence without the range
// branches, and j taken from the bits of the rounding sum t = 1.5 * 2^23 + j
// (exact for |j| < 2^22) instead of a float -> int conversion, so it returns
// gsx_expf(x) bit for bit there (j >= -126: the scale 2^j stays normal).
__device__ __forceinline__ float gsx_expf_neg(float x) {
  float t = fmaf(x, 1.44269502162933349609375f, 12582912.0f);
  float j = t - 12582912.0f;
  float r = fmaf(j, -0.693145751953125f, x);
  r = fmaf(j, -1.428606765330187045e-06f, r);
  float p = 1.98412698412698412e-04f;
  p = fmaf(p, r, 1.38888888888888889e-03f);
  p = fmaf(p, r, 8.33333333333333333e-03f);
  p = fmaf(p, r, 4.16666666666666667e-02f);
  p = fmaf(p, r, 1.66666666666666667e-01f);
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  const int ji = __float_as_int(t) - 0x4B400000;  // t = 12582912 + j
  return p * __int_as_float((ji + 127) << 23);
}

// gsx_expf for every x <= 0 and NaN (the raster's exponent -radial/2),
// without branches: equal to gsx_expf there bit for bit (+0 at and below
// -87, NaN for NaN).
__device__ __forceinline__ float gsx_expf_nonpos(float x) {
  const float e = gsx_expf_neg(fmaxf(x, -87.0f));
  return x > -87.0f ? e : (x != x ? x : 0.0f);
}

// gsx_expf_nonpos of two values at once, every floating-point step a paired
// float2 operation (FFMA2 / FADD2 / FMUL2 round each half exactly as the
// scalar instruction does), so each half equals gsx_expf_nonpos bit for bit.
__device__ __forceinline__ float2 gsx_expf_nonpos2(float2 x) {
  const float2 xc = make_float2(fmaxf(x.x, -87.0f), fmaxf(x.y, -87.0f));
  const float2 magic = make_float2(12582912.0f, 12582912.0f);
  const float2 t = __ffma2_rn(xc, make_float2(1.44269502162933349609375f, 1.44269502162933349609375f), magic);
  const float2 j = __fadd2_rn(t, make_float2(-12582912.0f, -12582912.0f));
  float2 r = __ffma2_rn(j, make_float2(-0.693145751953125f, -0.693145751953125f), xc);
  r = __ffma2_rn(j, make_float2(-1.428606765330187045e-06f, -1.428606765330187045e-06f), r);
  float2 p = make_float2(1.98412698412698412e-04f, 1.98412698412698412e-04f);
  p = __ffma2_rn(p, r, make_float2(1.38888888888888889e-03f, 1.38888888888888889e-03f));
  p = __ffma2_rn(p, r, make_float2(8.33333333333333333e-03f, 8.33333333333333333e-03f));
  p = __ffma2_rn(p, r, make_float2(4.16666666666666667e-02f, 4.16666666666666667e-02f));
  p = __ffma2_rn(p, r, make_float2(1.66666666666666667e-01f, 1.66666666666666667e-01f));
  p = __ffma2_rn(p, r, make_float2(0.5f, 0.5f));
  p = __ffma2_rn(p, r, make_float2(1.0f, 1.0f));
  p = __ffma2_rn(p, r, make_float2(1.0f, 1.0f));
  const int j0 = __float_as_int(t.x) - 0x4B400000, j1 = __float_as_int(t.y) - 0x4B400000;
  const float2 e = __fmul2_rn(p, make_float2(__int_as_float((j0 + 127) << 23), __int_as_float((j1 + 127) << 23)));
  return make_float2(x.x > -87.0f ? e.x : (x.x != x.x ? x.x : 0.0f),
                     x.y > -87.0f ? e.y : (x.y != x.y ? x.y : 0.0f));
}

__device__ __forceinline__ float gsx_sigmoidf(float x) {
  return 1.0f / (1.0f + gsx_expf(-x));
}

// float -> int32 truncation with saturation and NaN -> 0 (cvt.rzi.s32.f32).
__device__ __forceinline__ int32_t f2i_sat(float f) { return __float2int_rz(f); }

// Sphere-vs-frustum test of gs/src/include/kernels.h:156-170.
__device__ __forceinline__ bool sphere_in_frustum(float mx, float my, float mz,
                                                  float r, const float *normals,
                                                  const float *pts) {
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    float dx = mx - pts[3 * i], dy = my - pts[3 * i + 1], dz = mz - pts[3 * i + 2];
    float d = fmaf(dz, normals[3 * i + 2], fmaf(dy, normals[3 * i + 1], dx * normals[3 * i]));
    if (!(d > -r)) return false;
  }
  return true;
}

// ---- programmatic dependent launch ----------------------------------------
// A kernel launched by launch_pdl may be scheduled while the previous kernel
// on its stream is still finishing (its launch and CTA set-up overlap that
// kernel's last wave).  Every such kernel calls pdl_wait() before it reads or
// writes anything: the wait returns once the previous kernel has completed
// and its memory operations are visible, so the stream order of the results
// is unchanged.  pdl_trigger() right after the wait lets the next kernel be
// scheduled in turn.  Both are no-ops for a kernel launched without the
// attribute.
#ifndef GSX_PDL
#define GSX_PDL 1
#endif

__device__ __forceinline__ void pdl_wait() {
#if GSX_PDL
  asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}

__device__ __forceinline__ void pdl_trigger() {
#if GSX_PDL
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = GSX_PDL ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// ---- bulk copies (the TMA engine) and mbarriers ----------------------------
// cp.async.bulk global -> shared completing on an mbarrier; every wait on a
// barrier phase is bounded (kBulkWaitLimit polls), after which the caller
// flags an error instead of spinning on.
constexpr uint32_t kBulkWaitLimit = 1u << 20;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase `parity` of `bar`; false if it did not complete.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  for (uint32_t i = 0; i < kBulkWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes,
                                              uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}


// Host-side helpers (implemented in abi.cu).
void set_error(const char *fmt, ...);
void clear_error();  // empties this thread's gsx_last_error message
int cuda_status(cudaError_t e, const char *what);
// Ranges every binning entry point accepts: n and the key count in [0, 2^30),
// a positive tile grid of fewer than 2^31 tiles.
int check_binning_sizes(int64_t n, int64_t cap, int32_t nth, int32_t ntw);
// Counts kernel launches issued by this library (read by gsx_kernel_launch_count).
void count_launches(unsigned n);

// Launchers (each returns a GSX status).
int launch_cull_bsphere(int64_t n, const float *mean, const float *svec,
                        const float *normal, const float *pts, uint8_t *mask,
                        float thresh, cudaStream_t s);
int launch_project_forward(int64_t n, const float *mean, const float *qvec,
                           const float *log_scale, const float *alpha_logit,
                           const gsx_camera &cam, float frustum_radius,
                           float tile_radius, int32_t tile_w, int32_t tile_h,
                           int32_t scales_are_activated, float *mean2d,
                           float *cov2d, float *depth, float *alpha, int32_t *rect,
                           int32_t *counts, cudaStream_t s);
int launch_project_backward(int64_t n, const float *mean, const float *qvec,
                            const float *log_scale, const float *alpha_logit,
                            const gsx_camera &cam, const int32_t *counts,
                            const float *g_mean2d, const float *g_cov2d,
                            const float *g_alpha, float *g_mean, float *g_qvec,
                            float *g_logs, float *g_alpha_logit, int32_t flags, cudaStream_t s);

int launch_project_forward_batch(const gsx_batch_view *views, int32_t n_views, int64_t max_n,
                                 float frustum_radius, float tile_radius, float *mean2d,
                                 float *cov2d, float *depth, float *alpha, int32_t *rect,
                                 int32_t *counts, cudaStream_t s);
int launch_project_backward_batch(const gsx_batch_view *views, int32_t n_views, int64_t n,
                                  const int32_t *counts, const float *g_mean2d,
                                  const float *g_cov2d, const float *g_alpha, int32_t flags,
                                  cudaStream_t s);

// Opt-in per-Gaussian colours (colors.cu): rgb [n,3] from the direction
// camera centre -> mean; the backward overwrites g_sh [n,3,sh_stride] and adds
// the direction's share of the gradient into g_mean [n,3].
int launch_colors_forward(int64_t n, const float *mean, const float *sh, int sh_stride, int C,
                          const float *cam_pos_host, const int32_t *counts, float *rgb,
                          cudaStream_t s);
int launch_colors_backward(int64_t n, const float *mean, const float *sh, int sh_stride, int C,
                           const float *cam_pos_host, const int32_t *counts, const float *rgb,
                           const float *g_rgb, float *g_sh, float *g_mean, cudaStream_t s);

// Adaptive density control (densify.cu).
int launch_count_visible(int64_t n, const int32_t *counts, int32_t *cnt, cudaStream_t s);
int launch_accumulate_norm(int64_t n, const float *grad, int dim, const int32_t *counts,
                           float *accum, int reduce_max, cudaStream_t s);
int launch_classify(int64_t n, const float *accum, const int32_t *cnt, const float *log_scale,
                    float grad_thresh, float scale_thresh, int divide_by_count, uint8_t *cls,
                    cudaStream_t s);
int launch_rewrite(int64_t n, const uint8_t *cls, const int64_t *pos_stay, const int64_t *pos_clone,
                   const int64_t *pos_split, int64_t n_stay, int64_t n_clone, int64_t n_split,
                   const float *mean, const float *qvec, const float *log_scale, const float *sh,
                   int sh_len, const float *alpha_logit, float log_shrink, uint64_t seed,
                   float *o_mean, float *o_qvec, float *o_log_scale, float *o_sh, float *o_alpha,
                   cudaStream_t s);

// Training step (train.cu).
size_t loss_workspace_bytes(int H, int W);
int run_ssim_loss(const float *out, const float *gt, int H, int W, int win_size, float ssim_mult,
                  int l2, float *grad_out, float *partial_out, void *ws, cudaStream_t s);
int launch_adam(const gsx_adam_group *groups_dev, int n_groups, int64_t total,
                const int64_t *offsets_dev, cudaStream_t s);

struct RasterArgs {
  int64_t n, n_keys;  // Gaussians and list entries: bounds for start/end/ids
  int32_t width, height, tile_w, tile_h, n_tiles_w, n_tiles_h;
  int32_t sh_stride;
  int32_t batch;  // Gaussians per shared-memory batch (set by the launcher)
  float psx, psy, T_thresh;
  int32_t write_empty;
  const float *mean2d, *cov2d, *sh, *alpha;
  const int32_t *start, *end, *ids;
  const float *topleft, *c2w;
  float *out;
  // backward only
  const float *final_img, *grad_out;
  float *g_mean2d, *g_cov2d, *g_sh, *g_alpha;
  // batched passes: per-view table in device memory (nullptr for one view)
  const gsx_batch_view *views;
  int32_t n_views;
  int32_t vec_grads;  // g_mean2d 8-byte and g_cov2d 16-byte aligned (set by the launcher)
  // forward extras (single view): background colour composited behind the
  // Gaussians, per-pixel alpha (1 - final T) and depth (sum of T a G z)
  int32_t has_bg;
  float bg[3];
  const float *depth;  // per-item camera depth (needed for depth_out)
  float *alpha_out, *depth_out;
  // single view: CTA b renders tile tile_order[b] (a permutation of the tiles,
  // longest lists first); nullptr renders tile b
  const int32_t *tile_order;
  // raster passes: 1 = one pixel per thread, 2 = two (tiles made of 8x8
  // blocks only), 0 = two wherever possible
  int32_t pixels_per_thread;
  // work items (tiles) of the launch, set by the launcher; with work_counter
  // (a zeroed device word) the grid is persistent: resident CTAs claim the
  // items (tile_order[item] when given) one atomic at a time
  int64_t n_work;
  uint32_t *work_counter;
};
int launch_raster_forward(const RasterArgs &a, int C, cudaStream_t s);
// order[0..n_tiles) = the tiles by descending list length (end - start), in
// log-spaced length classes; the order within a class is unspecified.
int launch_tile_order(const int32_t *start, const int32_t *end, int32_t n_tiles, int32_t *order,
                      cudaStream_t s);
int launch_raster_backward(const RasterArgs &a, int C, cudaStream_t s);
// Per-Gaussian colours: a.sh = rgb [n,3] (a.sh_stride = 1); the backward adds
// dL/drgb into a.g_sh.
int launch_raster_forward_rgb(const RasterArgs &a, cudaStream_t s);
int launch_raster_backward_rgb(const RasterArgs &a, cudaStream_t s);
// Batched: a.views/a.n_views set, grid = total tiles (all views share the tile
// shape and SH order; the per-view fields of `a` are ignored).
int launch_raster_forward_batch(const RasterArgs &a, int C, int64_t total_tiles, cudaStream_t s);
int launch_raster_backward_batch(const RasterArgs &a, int C, int64_t total_tiles, cudaStream_t s);
// Sticky error bits of the raster kernels (synchronises `s`); clear != 0
// resets them.
int raster_status(uint32_t *flags, int clear, cudaStream_t s);
// One CTA waits on a barrier phase that cannot complete, for `limit` polls;
// sets the raster timeout bit and writes the polls made to polls_dev[0].
int raster_wait_selftest(uint32_t limit, uint32_t *polls_dev, cudaStream_t s);

// out[i] = gsx_expf (variant 0), gsx_expf_nonpos (1) or gsx_expf_nonpos2 on
// the pairs (x[2k], x[2k+1]) (2) of x[i], for i < n.
int exp_selftest(const float *x, int64_t n, float *out, int variant, cudaStream_t s);

// Binning.  rect_tl/rect_br point at int32 pairs with `rect_stride` ints per
// Gaussian (4 for packed [n,4] rects, 2 for separate [n,2] arrays).
size_t binning_workspace_bytes(int64_t n, int64_t cap, int64_t n_tiles);
int run_binning_async(int64_t n, const int32_t *rect_tl, const int32_t *rect_br,
                      int32_t rect_stride, const int32_t *counts, const float *depth,
                      int32_t n_tiles_w, int32_t n_tiles_h, int64_t capacity, int32_t *ids,
                      int32_t *start, int32_t *end, void *ws, size_t ws_bytes, cudaStream_t s,
                      const gsx_batch_view *views = nullptr, int32_t n_views = 0,
                      int64_t total_tiles = 0, int64_t max_view_tiles = 0);
int binning_status(const void *ws, int64_t n, int64_t capacity, int32_t n_tiles_w,
                   int32_t n_tiles_h, int64_t *n_keys_host, uint32_t *flags_host, cudaStream_t s);
int copy_binning_status_async(const void *ws, int64_t n, int64_t capacity, void *dst,
                              cudaStream_t s);
int decode_binning_status(unsigned long long total, uint32_t error_bits, int64_t capacity,
                          int32_t n_tiles_w, int32_t n_tiles_h);
size_t look_back_selftest_bytes();
int look_back_selftest(void *scratch, size_t bytes, uint32_t *error_host, cudaStream_t s);
int run_binning(int64_t n, const int32_t *rect_tl, const int32_t *rect_br,
                int32_t rect_stride, const int32_t *counts, const float *depth,
                int32_t n_tiles_w, int32_t n_tiles_h, int64_t capacity,
                int32_t *ids, int32_t *start, int32_t *end, int64_t *n_keys_host,
                void *ws, size_t ws_bytes, cudaStream_t s);

}  // namespace gsx
