// raster.cu -- tile-based front-to-back SH compositing, forward and backward.
//
// Reference behaviour restated (gs/src/include/vol_render_sh.h):
//   pixel position        :117-118, :213-214  topleft + (gx, gy) * pixel_size
//   SH view direction     :48-65  c2w read as float3 rows of the flat [3,4]
//                         array (rows 0..2 = floats 0-2, 3-5, 6-8), normalised
//   SH basis              shencoder.h:13-58 (C <= 4 used)
//   forward per pair      :120-168  T < thresh stops the pixel; a = min(alpha,
//                         .99); skip if a*G < 1/255; colour = sigmoid(sh . Y)
//   backward per pair     :295-350  same recompute; dL/dsh, dL/d(aG) through
//                         (final - out)/(1 - aG), 2D-Gaussian grads
//                         (kernels.h:394-418), dL/dalpha = P * G
//
// GB300 layout: one CTA per tile, one thread per pixel, each warp an 8x4
// block of pixels.  Each batch of the tile's sorted list is gathered once into
// shared memory and compacted to the Gaussians whose conservative skip box
// meets the tile; their SH rows arrive by cp.async.bulk (the TMA engine) on
// an mbarrier; all threads then read the records as broadcasts.  Each warp
// walks only the batch Gaussians whose skip box and skip ellipse meet its
// pixel block.  A CTA leaves the list as soon as every pixel has saturated
// (__syncthreads_and on the per-pixel stop flag), which changes no pixel: a
// stopped pixel takes no further Gaussian in the reference either.
//
// Arithmetic.  Everything that decides which pairs contribute -- the radial
// distance, the exponential G (gsx_expf), a*G < 1/255, the transmittance T --
// follows the operation sequence the CPU oracle restates, so those decisions
// are bit-identical.  The colour path is a smooth function of its inputs and
// uses the fast hardware forms: paired FMAs (two interleaved partial sums)
// for the SH dot products and ex2/rcp for the sigmoid; images agree with the
// oracle to ~1e-6.
//
// Backward.  Per contributing pair the thread forms the three SH weights
// w_ch and six scalar gradients.  The scalars are summed over the warp with a
// short butterfly.  The SH gradient of a Gaussian is the product
// sum_p w_ch(p) Y_k(p) over the warp's 32 pixels, so each warp stages the
// weights of up to five Gaussians as a 15x32 matrix and multiplies it with its
// 32x16 basis matrix on the tensor cores (mma.sync m16n8k8, TF32 split into
// high and low parts, three products, FP32 accumulation: ~2^-21 relative per
// product).  Warp results meet in shared memory (atomics), and the CTA issues
// one global atomic per (tile, Gaussian, value).
#include <cuda_fp16.h>

#include "gsx_internal.cuh"

namespace gsx {

// Sticky error bits of the raster kernels (read and cleared by
// raster_status); kRasterErrTimeout: a bulk-copy barrier wait gave up.
__device__ uint32_t g_raster_flags = 0;

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kRasterErrTimeout = 1u;  // bit of g_raster_flags

template <int C>
struct Sh {
  static constexpr int CC = C * C;
  static constexpr int CCP = (CC + 3) & ~3;  // per-channel smem stride
  static constexpr int GSH = 3 * CCP;        // smem floats per Gaussian
  static constexpr int NY2 = (CC + 1) / 2;   // basis as float2 pairs
};

template <int C>
__device__ __forceinline__ void sh_basis(const float *__restrict__ c2w, float px, float py,
                                         float *Y) {
  float d[3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
    d[r] = fmaf(c2w[3 * r + 2], 1.0f, fmaf(c2w[3 * r + 1], py, c2w[3 * r] * px));
  float len = sqrtf(fmaf(d[2], d[2], fmaf(d[1], d[1], d[0] * d[0])));
  float x = d[0] / len, y = d[1] / len, z = d[2] / len;
  float xy = x * y, xz = x * z, yz = y * z, x2 = x * x, y2 = y * y, z2 = z * z;
  Y[0] = 0.28209479177387814f;
  if (C <= 1) return;
  Y[1] = -0.48860251190291987f * y;
  Y[2] = 0.48860251190291987f * z;
  Y[3] = -0.48860251190291987f * x;
  if (C <= 2) return;
  Y[4] = 1.0925484305920792f * xy;
  Y[5] = -1.0925484305920792f * yz;
  Y[6] = fmaf(0.94617469575755997f, z2, -0.31539156525251999f);
  Y[7] = -1.0925484305920792f * xz;
  Y[8] = fmaf(0.54627421529603959f, x2, -(0.54627421529603959f * y2));
  if (C <= 3) return;
  Y[9] = (0.59004358992664352f * y) * fmaf(-3.0f, x2, y2);
  Y[10] = (2.8906114426405538f * xy) * z;
  Y[11] = (0.45704579946446572f * y) * fmaf(-5.0f, z2, 1.0f);
  Y[12] = (0.3731763325901154f * z) * fmaf(5.0f, z2, -3.0f);
  Y[13] = (0.45704579946446572f * x) * fmaf(-5.0f, z2, 1.0f);
  Y[14] = (1.4453057213202769f * z) * (x2 - y2);
  Y[15] = (0.59004358992664352f * x) * fmaf(3.0f, y2, -x2);
}

// sum_k sh[k] * Y[k] with paired FMAs over (even, odd) k; `s` is 16-byte
// aligned, Y2[j] = (Y[2j], Y[2j+1]).
template <int C>
__device__ __forceinline__ float sh_logit(const float *__restrict__ s, const float2 *Y2) {
  constexpr int CC = C * C;
  if constexpr (CC == 1) {
    return s[0] * Y2[0].x;
  } else {
    float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int k = 0; k + 3 < CC; k += 4) {
      const float4 q = *reinterpret_cast<const float4 *>(s + k);
      acc = __ffma2_rn(make_float2(q.x, q.y), Y2[k / 2], acc);
      acc = __ffma2_rn(make_float2(q.z, q.w), Y2[k / 2 + 1], acc);
    }
    float r = acc.x + acc.y;
    if constexpr (CC % 4 != 0) r = fmaf(s[CC - 1], Y2[CC / 2].x, r);  // CC = 9
    return r;
  }
}

__device__ __forceinline__ float fast_sigmoid(float x) {
  float e, r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(x * -1.4426950408889634f));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(1.0f + e));
  return r;
}

// radial distance of gs/src/include/kernels.h:172-187 (before the exp), for
// the pixel offset x = px - mean.x, y = py - mean.y.
__device__ __forceinline__ float radial_of(float4 cv, float x, float y) {
  float det = fmaf(cv.x, cv.w, -(cv.y * cv.z));
  float tmpx = fmaf(x, cv.w, -(y * cv.z));
  float tmpy = fmaf(-x, cv.y, y * cv.x);
  float radial = fmaf(tmpx, x, tmpy * y);
  radial = radial / det;
  if (radial < 0.0f) radial = 1000.0f;
  return radial;
}

// For radial > 12, exp(-radial/2) < 0.0025, so a*G < 1/255 for every finite
// a <= 0.99: the pair is skipped without evaluating the exponential.  (a is
// never NaN after fminf; a == -inf would give NaN at G == 0 and is excluded.)
__device__ __forceinline__ bool surely_skipped(float radial, float a) {
  return radial > 12.0f && a != -__int_as_float(0x7f800000);
}

// Per-CTA view of the work: which tile of which image, and where the view's
// scene and image live.  One view: everything comes from the kernel
// arguments.  Batched: the global tile number selects the view from the
// device table (binary search over the tile offsets).
struct ViewCtx {
  int gtile;  // tile index in start/end (global over the batch)
  int tile;   // tile index within the view's image
  int n_tiles_w, tile_w, tile_h, width, height;
  float psx, psy;
  const float *topleft, *c2w;
  const float *sh;
  int sh_stride;
  int64_t item_lo, item_hi;  // items of this view: [item_lo, item_hi)
  float *out;
  const float *final_img, *grad_out;
  float *g_sh;
  int write_empty;
};

// Work items of a raster launch: one per tile.  Without a work counter CTA b
// takes item b; with one (a persistent grid of resident CTAs) every CTA
// claims items in turn through one atomic each, until a.n_work are taken.
// Returns -1 when the CTA has no further item.  CTA-uniform.
template <bool PERSIST>
__device__ __forceinline__ int64_t claim_work(const RasterArgs &a, int *s_work, bool first) {
  if constexpr (!PERSIST) return first ? (int64_t)blockIdx.x : -1;
  __syncthreads();  // the previous tile's shared memory is no longer read
  if (threadIdx.x == 0) *s_work = (int)atomicAdd(a.work_counter, 1u);
  __syncthreads();
  const int64_t w = *s_work;
  return w < a.n_work ? w : -1;
}

// The tile of work item `work`: tile_order[work] (longest lists first) or the
// item itself; an entry outside [0, n_work) renders nothing (gtile = -1).
template <bool BATCHED>
__device__ __forceinline__ ViewCtx make_ctx(const RasterArgs &a, int64_t work) {
  ViewCtx c;
  int64_t g = a.tile_order ? (int64_t)a.tile_order[work] : work;
  if (g < 0 || g >= a.n_work) g = -1;
  c.gtile = (int)g;
  if (g < 0) return c;
  if constexpr (!BATCHED) {
    c.tile = c.gtile;
    c.n_tiles_w = a.n_tiles_w;
    c.tile_w = a.tile_w;
    c.tile_h = a.tile_h;
    c.width = a.width;
    c.height = a.height;
    c.psx = a.psx;
    c.psy = a.psy;
    c.topleft = a.topleft;
    c.c2w = a.c2w;
    c.sh = a.sh;
    c.sh_stride = a.sh_stride;
    c.item_lo = 0;
    c.item_hi = a.n;
    c.out = a.out;
    c.final_img = a.final_img;
    c.grad_out = a.grad_out;
    c.g_sh = a.g_sh;
    c.write_empty = a.write_empty;
  } else {
    const int64_t gt = g;
    int lo = 0, hi = a.n_views - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (a.views[mid].tile_offset <= gt) lo = mid;
      else hi = mid - 1;
    }
    const gsx_batch_view &v = a.views[lo];
    c.tile = (int)(gt - v.tile_offset);
    c.n_tiles_w = v.n_tiles_w;
    c.tile_w = v.tile_w;
    c.tile_h = v.tile_h;
    c.width = v.cam.width;
    c.height = v.cam.height;
    c.psx = v.pixel_size_x;
    c.psy = v.pixel_size_y;
    c.topleft = v.topleft;
    c.c2w = v.cam.c2w;
    c.sh = v.sh;
    c.sh_stride = v.sh_stride;
    c.item_lo = v.item_offset;
    c.item_hi = v.item_offset + v.n_gaussians;
    c.out = v.out;
    c.final_img = v.out;
    c.grad_out = v.grad_out;
    c.g_sh = v.g_sh;
    c.write_empty = v.write_empty_tiles;
  }
  return c;
}

// Length of a tile's list; 0 for empty tiles (start == -1, as the reference
// marks them) and for ranges that do not fit in [0, n_keys).
__device__ __forceinline__ int tile_list_length(const RasterArgs &a, int gtile, int s0) {
  if (s0 < 0) return 0;
  const int e = a.end[gtile];
  if (e < s0 || (int64_t)e > a.n_keys) return 0;
  return e - s0;
}

// Pixel of thread t: warps cover 8x4 blocks when the tile allows it (a
// compact footprint means fewer warps per small Gaussian), else rows.
__device__ __forceinline__ void pixel_of(const ViewCtx &c, int t, int &gx, int &gy) {
  int lx, ly;
  if ((c.tile_w & 7) == 0 && (c.tile_h & 3) == 0) {
    const int w = t >> 5, l = t & 31, bpr = c.tile_w >> 3;
    lx = (w % bpr) * 8 + (l & 7);
    ly = (w / bpr) * 4 + (l >> 3);
  } else {
    lx = t % c.tile_w;
    ly = t / c.tile_w;
  }
  gx = (c.tile % c.n_tiles_w) * c.tile_w + lx;
  gy = (c.tile / c.n_tiles_w) * c.tile_h + ly;
}

// Normalised coordinates of the first and last pixel centres of a tile that
// lie inside the image (computed like the pixel positions themselves).
__device__ __forceinline__ void tile_bounds(const ViewCtx &c, float &x0, float &x1, float &y0,
                                            float &y1) {
  const int gx0 = (c.tile % c.n_tiles_w) * c.tile_w, gy0 = (c.tile / c.n_tiles_w) * c.tile_h;
  const int gx1 = min(gx0 + c.tile_w, c.width) - 1, gy1 = min(gy0 + c.tile_h, c.height) - 1;
  x0 = fmaf((float)gx0, c.psx, c.topleft[0]);
  x1 = fmaf((float)gx1, c.psx, c.topleft[0]);
  y0 = fmaf((float)gy0, c.psy, c.topleft[1]);
  y1 = fmaf((float)gy1, c.psy, c.topleft[1]);
  if (x0 > x1) { const float tmp = x0; x0 = x1; x1 = tmp; }
  if (y0 > y1) { const float tmp = y0; y0 = y1; y1 = tmp; }
}

struct SmemLayout {
  float4 *cov;
  float2 *mean;
  float2 *box;  // half-extents of the region where the pair may contribute
  float *alpha;
  int *ids;
  float *inv_det;  // 1 / det(cov), backward only
  float *zdep;     // camera depth, forward with a depth map only
  float *rq;       // skip radius R of the ellipse test (inf: no ellipse test)
  float *sh;
};

constexpr int kRecordFloats = 13;  // floats of per-Gaussian records per batch slot

// Shared-memory layout of one batch of B Gaussians (B a multiple of 4):
// kRecordFloats*B floats of records followed by the SH rows (16-byte aligned).
template <int C>
__device__ __forceinline__ SmemLayout carve(float *smem, int B) {
  SmemLayout L;
  L.cov = reinterpret_cast<float4 *>(smem);
  L.mean = reinterpret_cast<float2 *>(smem + 4 * B);
  L.box = reinterpret_cast<float2 *>(smem + 6 * B);
  L.alpha = smem + 8 * B;
  L.ids = reinterpret_cast<int *>(smem + 9 * B);
  L.inv_det = smem + 10 * B;
  L.zdep = smem + 11 * B;
  L.rq = smem + 12 * B;
  L.sh = smem + kRecordFloats * B;
  return L;
}

__device__ __forceinline__ float inf_f() { return __int_as_float(0x7f800000); }

// Conservative skip region of one Gaussian.  With a = min(alpha, .99), a pair
// is skipped by the reference when a * exp(-radial/2) < 1/255, i.e. whenever
// radial > R_a = 2 ln(255 a).  For a well-conditioned covariance (both
// diagonal entries positive, det > 1e-2 * c0 * c3, all finite) the float
// radial differs from the exact quadratic form by far less than 1e-3
// relative, so every pixel outside the ellipse x^T S^-1 x <= 1.01 R_a + 0.05
// is skipped; that ellipse lies inside the box |dx| <= sqrt(R c0),
// |dy| <= sqrt(R c3), widened by 1 % more.  drop = the Gaussian is skipped by
// every pixel (a < 1/255 with a finite, non-negative G).  Anything else gets
// an infinite box and takes the exact per-pixel path.  `rq` receives R for
// the ellipse test of ellipse_meets_block when the two off-diagonal entries
// agree (as a projected covariance's do up to rounding), else +inf.
__device__ __forceinline__ float2 skip_box(float4 cv, float2 m, float a, bool &drop, float &rq) {
  drop = false;
  rq = inf_f();
  const bool finite = isfinite(cv.x) && isfinite(cv.y) && isfinite(cv.z) && isfinite(cv.w) &&
                      isfinite(m.x) && isfinite(m.y);
  const float det = fmaf(cv.x, cv.w, -(cv.y * cv.z));
  const bool good = finite && cv.x > 0.0f && cv.w > 0.0f && det > 1e-2f * (cv.x * cv.w);
  if (!good || !(a == a)) return make_float2(inf_f(), inf_f());
  if (a < kMinRenderAlpha) {
    drop = true;
    return make_float2(0.0f, 0.0f);
  }
  const float R = fmaxf(2.0f * logf(255.0f * a), 0.0f) * 1.01f + 0.05f;
  if (fabsf(cv.y - cv.z) <= 1e-4f * sqrtf(cv.x * cv.w)) rq = R;
  return make_float2(sqrtf(R * cv.x) * 1.01f + 1e-6f, sqrtf(R * cv.w) * 1.01f + 1e-6f);
}

// Conservative test that some point of the block [blk.x, blk.y] x [blk.z,
// blk.w] (the warp's pixel centres) lies inside the ellipse where the pair can
// reach 1/255: min over the block of the quadratic form of the radial,
// (c3 x^2 - (c1 + c2) x y + c0 y^2) / det, is at most R.  The form is positive
// definite for the covariances skip_box hands an R (c0, c3 > 0, det > 1e-2
// c0 c3, c1 ~ c2), so when the centre lies outside the block the minimum is on
// its boundary, found per edge at the clamped stationary point.  Float error
// of the form is far below the 1 % widening of R; an extra 0.1 % is added,
// which also covers the approximate division of the stationary point (the
// form is flat there: an offset d raises it by c d^2, relative 2^-40 or less).
__device__ __forceinline__ bool ellipse_meets_block(float4 cv, float2 m, float R, float4 blk) {
  const float X0 = blk.x - m.x, X1 = blk.y - m.x, Y0 = blk.z - m.y, Y1 = blk.w - m.y;
  if (X0 <= 0.0f && X1 >= 0.0f && Y0 <= 0.0f && Y1 >= 0.0f) return true;
  const float A = cv.w, Cc = cv.x, H = 0.5f * (cv.y + cv.z);
  const float det = fmaf(cv.x, cv.w, -(cv.y * cv.z));
  const float lim = R * det * 1.001f;
  float best = inf_f();
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    const float X = e ? X1 : X0;
    const float y = fminf(fmaxf(__fdividef(H * X, Cc), Y0), Y1);
    best = fminf(best, fmaf(A * X, X, fmaf(-2.0f * H * X, y, Cc * y * y)));
    const float Y = e ? Y1 : Y0;
    const float x = fminf(fmaxf(__fdividef(H * Y, A), X0), X1);
    best = fminf(best, fmaf(A * x, x, fmaf(-2.0f * H * x, Y, Cc * Y * Y)));
  }
  return best <= lim;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned lt;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
  return lt;
}

// ---- bulk-copy (TMA engine) staging of the SH rows -------------------------
// A batch's SH rows are copied global -> shared with cp.async.bulk, one copy
// per kept Gaussian (or per channel when the rows are strided), completing on
// one mbarrier per CTA (helpers in gsx_internal.cuh).  Thread 0 arms the
// barrier with the batch's byte total; the phase flips once per batch.

// Diagnostic of the bounded wait: one CTA polls a barrier phase that cannot
// complete (two arrivals expected, one made, no copies), gives up after
// `limit` polls and sets the same error bit as a raster whose bulk-copy wait
// gave up.  out[0] = polls made by thread 0.
__global__ void bounded_wait_selftest_kernel(uint32_t limit, uint32_t *out) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 2;" ::"r"(smem_u32(&bar)) : "memory");
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&bar)) : "memory");
  }
  __syncthreads();
  uint32_t i = 0;
  bool ok = false;
  for (; i < limit && !ok; ++i) ok = mbar_try_wait(&bar, 0);
  if (!ok) atomicOr(&g_raster_flags, kRasterErrTimeout);
  if (threadIdx.x == 0) out[0] = i;
}

// The SH rows of this CTA's scene can be bulk-copied: every copy starts on a
// 16-byte boundary and moves a multiple of 16 bytes (C*C and the row stride
// multiples of 4 floats, base 16-byte aligned).
template <int C>
__device__ __forceinline__ bool sh_bulk_ok(const float *sh, int sh_stride) {
  return (C * C) % 4 == 0 && (sh_stride & 3) == 0 &&
         (reinterpret_cast<uintptr_t>(sh) & 15) == 0;
}

// Gather one batch of the tile's list into shared memory, keeping only the
// Gaussians whose skip box meets the tile's pixel centres (in list order).
// Requires nb <= blockDim.x.  Returns the number kept, or -1 (for the whole
// CTA) if a bulk-copy wait gave up.  INV_DET also stores 1 / det(cov) (the
// same operation the per-pair code would do).  When the SH rows allow it
// (sh_bulk_ok), each kept Gaussian's rows arrive by cp.async.bulk on `bar`
// (phase `parity`, initialised by the kernel); otherwise the CTA copies them
// with ordinary loads.
template <int C, bool INV_DET, bool DEPTH = false>
__device__ __forceinline__ int load_batch(const RasterArgs &a, const ViewCtx &ctx,
                                          const SmemLayout &L, int first, int nb, int t, int nthr,
                                          float tx0, float tx1, float ty0, float ty1,
                                          int *s_wcount, uint64_t *bar, uint32_t parity) {
  constexpr int CC = Sh<C>::CC, CCP = Sh<C>::CCP, GSH = Sh<C>::GSH;
  const int lane = t & 31, warp = t >> 5, nwarps = nthr >> 5;
  const bool bulk = sh_bulk_ok<C>(ctx.sh, ctx.sh_stride);  // CTA-uniform
  bool keep = false;
  int id = -1;
  float2 mm = make_float2(0.0f, 0.0f), box = make_float2(0.0f, 0.0f);
  float4 cv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  float al = 0.0f, rq = 0.0f;
  if (t < nb) {
    id = a.ids[first + t];
    if (id >= ctx.item_lo && id < ctx.item_hi) {
      const float *m = a.mean2d + 2 * (int64_t)id;
      const float *c = a.cov2d + 4 * (int64_t)id;
      mm = make_float2(m[0], m[1]);
      cv = make_float4(c[0], c[1], c[2], c[3]);
      al = fminf(a.alpha[id], 0.99f);
      bool drop;
      box = skip_box(cv, mm, al, drop, rq);
      keep = !drop && !(mm.x + box.x < tx0) && !(mm.x - box.x > tx1) && !(mm.y + box.y < ty0) &&
             !(mm.y - box.y > ty1);
    }
    // ids outside the view's items are dropped: no reads of the caller's arrays
  }
  const unsigned ballot = __ballot_sync(kFull, keep);
  if (lane == 0) s_wcount[warp] = __popc(ballot);
  __syncthreads();
  int before = 0, total = 0;
  for (int w = 0; w < nwarps; ++w) {
    const int c = s_wcount[w];
    before += (w < warp) ? c : 0;
    total += c;
  }
  if (bulk && t == 0) mbar_arrive_expect_tx(bar, (uint32_t)(total * 3 * CC * sizeof(float)));
  if (keep) {
    const int pos = before + __popc(ballot & lanemask_lt());
    L.ids[pos] = id;
    L.mean[pos] = mm;
    L.cov[pos] = cv;
    L.alpha[pos] = al;
    L.box[pos] = box;
    L.rq[pos] = rq;
    if constexpr (INV_DET) L.inv_det[pos] = 1.0f / fmaf(cv.x, cv.w, -(cv.y * cv.z));
    if constexpr (DEPTH) {
      if (a.depth_out) L.zdep[pos] = a.depth[id];
    }
    if (bulk) {
      // the previous batch's reads of this slot finished before the barrier
      // above; order them before the async-proxy writes
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      const int64_t g = (int64_t)id - ctx.item_lo;
      const float *src = ctx.sh + g * 3 * ctx.sh_stride;
      float *dst = L.sh + pos * GSH;
      if (ctx.sh_stride == CC) {
        bulk_copy_g2s(dst, src, 3 * CC * sizeof(float), bar);
      } else {
#pragma unroll
        for (int ch = 0; ch < 3; ++ch)
          bulk_copy_g2s(dst + ch * CCP, src + ch * ctx.sh_stride, CC * sizeof(float), bar);
      }
    }
  }
  if (bulk) {
    bool ok = mbar_wait_bounded(bar, parity);
    if (!ok) {
      atomicOr(&g_raster_flags, kRasterErrTimeout);
      ok = mbar_wait_bounded(bar, parity);  // the copies may still land: wait once more
    }
    // records visible to all threads; the CTA leaves together if any wait gave up
    return __syncthreads_or(!ok) ? -1 : total;
  }
  __syncthreads();
  const int count = total * 3 * CC;
  for (int f = t; f < count; f += nthr) {
    int j = f / (3 * CC);
    int rem = f - j * (3 * CC);
    int ch = rem / CC;
    int k = rem - ch * CC;
    const int64_t g = (int64_t)L.ids[j] - ctx.item_lo;  // Gaussian within the view's scene
    L.sh[j * GSH + ch * CCP + k] = ctx.sh[(g * 3 + ch) * ctx.sh_stride + k];
  }
  __syncthreads();
  return total;
}

// Bounds of the pixel centres of this warp's block (min/max over its lanes).
__device__ __forceinline__ float4 warp_block(float px, float py) {
  float x0 = px, x1 = px, y0 = py, y1 = py;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    x0 = fminf(x0, __shfl_xor_sync(kFull, x0, o));
    x1 = fmaxf(x1, __shfl_xor_sync(kFull, x1, o));
    y0 = fminf(y0, __shfl_xor_sync(kFull, y0, o));
    y1 = fmaxf(y1, __shfl_xor_sync(kFull, y1, o));
  }
  return make_float4(x0, x1, y0, y1);
}

// This warp's list of the batch Gaussians (batch positions, in order) whose
// skip box, and skip ellipse where there is one, meet the warp's pixel
// block; the others are skipped by every lane of the warp, so leaving them
// out changes nothing.  All lanes call it.
__device__ __forceinline__ int warp_list(const SmemLayout &L, int nk, float4 blk, int *wl,
                                         int lane) {
  int cnt = 0;
  for (int c = 0; c < nk; c += 32) {
    const int i = c + lane;
    bool hit = false;
    if (i < nk) {
      const float2 m = L.mean[i], h = L.box[i];
      hit = !(m.x + h.x < blk.x) && !(m.x - h.x > blk.y) && !(m.y + h.y < blk.z) &&
            !(m.y - h.y > blk.w);
      if (hit) {
        const float R = L.rq[i];
        if (R < inf_f()) hit = ellipse_meets_block(L.cov[i], m, R, blk);
      }
    }
    const unsigned b = __ballot_sync(kFull, hit);
    if (hit) wl[cnt + __popc(b & lanemask_lt())] = i;
    cnt += __popc(b);
  }
  __syncwarp();
  return cnt;
}

template <int C>
__device__ __forceinline__ void pack_basis(const float *Y, float2 *Y2) {
  constexpr int CC = Sh<C>::CC;
#pragma unroll
  for (int j = 0; j < Sh<C>::NY2; ++j)
    Y2[j] = make_float2(Y[2 * j], 2 * j + 1 < CC ? Y[(2 * j + 1) < CC ? 2 * j + 1 : 0] : 0.0f);
}

// EXTRAS: background colour and alpha / depth maps (single view only).
// RGB: per-Gaussian colours (an opt-in mode; the reference evaluates SH per
// pixel): `sh` holds rgb [n,3] as C = 1 rows, the basis is the constant 1
// and the colour is the stored value itself.
template <int C, int MAXT, bool BATCHED, bool EXTRAS, bool RGB = false, bool PERSIST = false>
__global__ void __launch_bounds__(MAXT) raster_forward_kernel(const RasterArgs a) {
  constexpr int GSH = Sh<C>::GSH, CCP = Sh<C>::CCP;
  extern __shared__ float4 smem4[];
  __shared__ int s_wcount[32];
  __shared__ uint64_t s_bar;  // bulk-copy barrier of the SH rows
  __shared__ int s_work;
  const int nthr = blockDim.x;
  const int B = a.batch;
  SmemLayout L = carve<C>(reinterpret_cast<float *>(smem4), B);
  int *wl = reinterpret_cast<int *>(L.sh + B * GSH) + (threadIdx.x >> 5) * B;  // [nwarps][B]

  if (PERSIST && threadIdx.x == 0) mbar_init(&s_bar);  // once per CTA, before any tile's first wait
  // bulk-copy phases completed by this CTA: the barrier's parity across the
  // tiles of a persistent grid (one tile per CTA: the batch index's parity)
  uint32_t nphase = 0;
  // one tile; false when the CTA must stop (a bulk-copy wait gave up)
  auto run_tile = [&](int64_t work) -> bool {
    const ViewCtx ctx = make_ctx<BATCHED>(a, work);
    if (ctx.gtile < 0) return true;  // CTA-uniform: not a tile of the grid
    if (!PERSIST && threadIdx.x == 0 && sh_bulk_ok<C>(ctx.sh, ctx.sh_stride))
      mbar_init(&s_bar);  // ordered before use by the batch loop's first barrier
    const int t = threadIdx.x, lane = t & 31;
    int gx, gy;
    pixel_of(ctx, t, gx, gy);
    const bool inside = t < ctx.tile_w * ctx.tile_h && gx < ctx.width && gy < ctx.height;
    const int s0 = a.start[ctx.gtile];
    const int n = tile_list_length(a, ctx.gtile, s0);
    if (n <= 0) {
      if (ctx.write_empty && inside) {
        const int64_t pix = (int64_t)gy * ctx.width + gx;
        float *dst = ctx.out + 3 * pix;
        const bool bg = EXTRAS && a.has_bg;
        dst[0] = bg ? a.bg[0] : 0.0f;
        dst[1] = bg ? a.bg[1] : 0.0f;
        dst[2] = bg ? a.bg[2] : 0.0f;
        if constexpr (EXTRAS) {
          if (a.alpha_out) a.alpha_out[pix] = 0.0f;
          if (a.depth_out) a.depth_out[pix] = 0.0f;
        }
      }
      return true;
    }
    const float px = fmaf((float)gx, ctx.psx, ctx.topleft[0]);
    const float py = fmaf((float)gy, ctx.psy, ctx.topleft[1]);
    float2 Y2[Sh<C>::NY2];
    {
      float Y[Sh<C>::CC];
      if constexpr (RGB) Y[0] = 1.0f;
      else sh_basis<C>(ctx.c2w, px, py, Y);
      pack_basis<C>(Y, Y2);
    }
    float o0 = 0.0f, o1 = 0.0f, o2 = 0.0f, T = 1.0f, dsum = 0.0f;
    const bool want_depth = EXTRAS && a.depth_out != nullptr;
    const float thr = a.T_thresh;
    bool done = !inside;
    float tx0, tx1, ty0, ty1;
    tile_bounds(ctx, tx0, tx1, ty0, ty1);
    const float4 blk = warp_block(px, py);

    for (int base = 0; base < n; base += B) {
      if (__syncthreads_and(done)) break;
      const int nb = min(B, n - base);
      const int nk = load_batch<C, false, EXTRAS>(a, ctx, L, s0 + base, nb, t, nthr, tx0, tx1, ty0,
                                                  ty1, s_wcount, &s_bar, PERSIST ? (nphase & 1u) : ((uint32_t)(base / B) & 1u));
      if (nk < 0) return false;  // flagged in g_raster_flags
      if (PERSIST && sh_bulk_ok<C>(ctx.sh, ctx.sh_stride)) ++nphase;
      const int nw = __all_sync(kFull, done) ? 0 : warp_list(L, nk, blk, wl, lane);
      if (!done) {
        for (int j = 0; j < nw; ++j) {
          const int i = wl[j];
          if (T < thr) {
            done = true;
            break;
          }
          const float2 m = L.mean[i];
          const float2 h = L.box[i];
          const float x = px - m.x, y = py - m.y;
          if (fabsf(x) > h.x || fabsf(y) > h.y) continue;
          const float al = L.alpha[i];
          const float radial = radial_of(L.cov[i], x, y);
          if (surely_skipped(radial, al)) continue;
          const float G = gsx_expf_nonpos(-0.5f * radial);
          float coeff = al * T;
          coeff = coeff * G;
          if (al * G < kMinRenderAlpha) continue;
          if (isnan(coeff)) coeff = 0.0f;
          const float *s = L.sh + i * GSH;
          float y0, y1, y2;
          if constexpr (RGB) {
            y0 = s[0];
            y1 = s[CCP];
            y2 = s[2 * CCP];
          } else {
            y0 = fast_sigmoid(sh_logit<C>(s, Y2));
            y1 = fast_sigmoid(sh_logit<C>(s + CCP, Y2));
            y2 = fast_sigmoid(sh_logit<C>(s + 2 * CCP, Y2));
          }
          // coeff is finite here, so y * coeff is NaN exactly when y is; fmaxf
          // returns its non-NaN operand and y >= 0, so this is the reference's
          // `if isnan(y * coeff) y = 0`
          y0 = fmaxf(y0, 0.0f);
          y1 = fmaxf(y1, 0.0f);
          y2 = fmaxf(y2, 0.0f);
          o0 = fmaf(coeff, y0, o0);
          o1 = fmaf(coeff, y1, o1);
          o2 = fmaf(coeff, y2, o2);
          if constexpr (EXTRAS) {
            if (want_depth) dsum = fmaf(coeff, L.zdep[i], dsum);
          }
          T = T * fmaf(-al, G, 1.0f);
        }
        if (T < thr) done = true;
      }
    }
    if (inside) {
      const int64_t pix = (int64_t)gy * ctx.width + gx;
      if (EXTRAS && a.has_bg) {  // what the Gaussians leave of the ray sees the background
        o0 = fmaf(T, a.bg[0], o0);
        o1 = fmaf(T, a.bg[1], o1);
        o2 = fmaf(T, a.bg[2], o2);
      }
      float *dst = ctx.out + 3 * pix;
      dst[0] = o0;
      dst[1] = o1;
      dst[2] = o2;
      if constexpr (EXTRAS) {
        if (a.alpha_out) a.alpha_out[pix] = 1.0f - T;
        if (want_depth) a.depth_out[pix] = dsum;
      }
    }
    return true;
  };
  if constexpr (PERSIST) {
    for (int64_t work = claim_work<true>(a, &s_work, true); work >= 0;
         work = claim_work<true>(a, &s_work, false))
      if (!run_tile(work)) return;
  } else {
    run_tile(blockIdx.x);
  }
}

// Vector reductions into global memory (red.global.add.v{2,4}.f32, sm_90+):
// the address must be 8- / 16-byte aligned.
__device__ __forceinline__ void red_add_v4(float *dst, float4 v) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst), "f"(v.x), "f"(v.y),
               "f"(v.z), "f"(v.w)
               : "memory");
}

__device__ __forceinline__ void red_add_v2(float *dst, float2 v) {
  asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(dst), "f"(v.x), "f"(v.y) : "memory");
}

// Sum of six per-lane values over the warp: reduce-scatter over offsets 16,
// 8, 4 (eight slots, two spare), then a butterfly over 2 and 1.  Afterwards
// lanes 4j hold the warp sum of value j.
__device__ __forceinline__ float warp_sum6(const float (&sc)[6], int lane) {
  float v[8] = {sc[0], sc[1], sc[2], sc[3], sc[4], sc[5], 0.0f, 0.0f};
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    const int o = 16 >> s;
    const int half = 4 >> s;
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int k = 0; k < half; ++k) {
      const float send = up ? v[k] : v[k + half];
      const float keep = up ? v[k + half] : v[k];
      v[k] = keep + __shfl_xor_sync(kFull, send, o);
    }
  }
  float r = v[0];
  r += __shfl_xor_sync(kFull, r, 2);
  r += __shfl_xor_sync(kFull, r, 1);
  return r;
}

__device__ __forceinline__ void split_tf32(float x, uint32_t &hi, uint32_t &lo) {
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hi) : "f"(x));
  const float rest = x - __uint_as_float(hi);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lo) : "f"(rest));
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr int kSlots = 5;     // Gaussians per warp matrix product (15 of 16 rows)
constexpr int kWStride = 36;  // row stride of the 16 x 32 weight matrix (bank-conflict free)
constexpr int kYStride = 36;  // row stride of the basis, stored k-major: 16 rows of 32 pixels
                              // (conflict-free both for the per-pixel writes and the
                              // B-fragment reads: bank = 4 g + tq + const)

// Per-Gaussian gradient record in shared memory (NV floats, 16-byte
// aligned): mean2d (0, 1), cov2d entries 0, 1 = 2, 3 (2, 3, 4), alpha (5),
// two spare, then 3 SH channels from float kShOff with a channel stride that
// keeps each channel 16-byte aligned and the three channels' atomics of one
// mma fragment on distinct banks (20 for C = 4: windows 8-15, 28-35, 16-23).
constexpr int kShOff = 8;
template <int C>
struct Grad {
  static constexpr int CC = C * C;
  // per-channel stride of the SH-gradient accumulators: C*C rounded up to 4
  // (a padded stride of 20 at C*C = 16 was measured slower: the smaller record
  // lets the two-pixel backward hold 48-Gaussian batches at four CTAs per SM)
  static constexpr int CSTR = (CC + 3) & ~3;
  static constexpr int NV = kShOff + 3 * CSTR;
};

// SH gradients of the staged Gaussians: D[r][k] = sum_p W[r][p] * Y[p][k] for
// rows r = 3*slot + channel, added into the batch accumulators.
template <int C>
__device__ __forceinline__ void flush_sh_group(const float *Ws, const float *Ys, const int *slots,
                                               int nslot, float *s_grad, int lane) {
  constexpr int CC = Sh<C>::CC;
  constexpr int NT = (CC + 7) / 8;
  constexpr int NV = Grad<C>::NV, CSTR = Grad<C>::CSTR;
  const int g = lane >> 2, tq = lane & 3;
  float d[NT][4];
#pragma unroll
  for (int nt = 0; nt < NT; ++nt) d[nt][0] = d[nt][1] = d[nt][2] = d[nt][3] = 0.0f;
#pragma unroll
  for (int ks = 0; ks < 4; ++ks) {
    uint32_t ah[4], al[4];
    split_tf32(Ws[g * kWStride + 8 * ks + tq], ah[0], al[0]);
    split_tf32(Ws[(g + 8) * kWStride + 8 * ks + tq], ah[1], al[1]);
    split_tf32(Ws[g * kWStride + 8 * ks + tq + 4], ah[2], al[2]);
    split_tf32(Ws[(g + 8) * kWStride + 8 * ks + tq + 4], ah[3], al[3]);
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
      uint32_t b0h, b0l, b1h, b1l;
      split_tf32(Ys[(8 * nt + g) * kYStride + 8 * ks + tq], b0h, b0l);
      split_tf32(Ys[(8 * nt + g) * kYStride + 8 * ks + tq + 4], b1h, b1l);
      mma_tf32(d[nt], ah, b0h, b1h);
      mma_tf32(d[nt], ah, b0l, b1l);
      mma_tf32(d[nt], al, b0h, b1h);
    }
  }
  const int rows = 3 * nslot;
#pragma unroll
  for (int nt = 0; nt < NT; ++nt)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int r = g + ((e & 2) ? 8 : 0);
      const int k = 8 * nt + 2 * tq + (e & 1);
      if (r < rows && k < CC && d[nt][e] != 0.0f) {
        const int slot = r / 3, ch = r - 3 * slot;
        atomicAdd(&s_grad[slots[slot] * NV + kShOff + ch * CSTR + k], d[nt][e]);
      }
    }
}

// Adds the batch's per-Gaussian accumulators (s_grad, kept Gaussians whose
// s_touched is set) into the global gradients: one vector reduction per chunk
// of a record -- mean2d (v2), cov2d (v4, entries 1 and 2 both get dL/dcov01 as
// the reference writes them), alpha, and the SH channels in 4-float chunks.
// Each chunk is set back to zero once read, so the accumulators need no
// clearing pass per batch (only touched records are ever written).
template <int C>
__device__ __forceinline__ void fold_batch_grads(const RasterArgs &a, const ViewCtx &ctx,
                                                 const SmemLayout &L, float *s_grad,
                                                 const int *s_touched, int nk, int t, int nthr) {
  constexpr int CC = Sh<C>::CC, NV = Grad<C>::NV;
  constexpr int NCH = Grad<C>::CSTR / 4;
  constexpr int NCHUNK = 3 + 3 * NCH;
  for (int f = t; f < nk * NCHUNK; f += nthr) {
    const int j = f / NCHUNK, c = f - j * NCHUNK;
    if (!s_touched[j]) continue;
    float *rec = s_grad + j * NV;
    const int64_t id = L.ids[j];
    if (c == 0) {
      const float2 v = *reinterpret_cast<const float2 *>(rec);
      *reinterpret_cast<float2 *>(rec) = make_float2(0.0f, 0.0f);
      if (a.vec_grads) {
        if (v.x != 0.0f || v.y != 0.0f) red_add_v2(a.g_mean2d + 2 * id, v);
      } else {
        if (v.x != 0.0f) atomicAdd(a.g_mean2d + 2 * id, v.x);
        if (v.y != 0.0f) atomicAdd(a.g_mean2d + 2 * id + 1, v.y);
      }
    } else if (c == 1) {
      const float4 v = make_float4(rec[2], rec[3], rec[3], rec[4]);
      rec[2] = rec[3] = rec[4] = 0.0f;
      if (a.vec_grads) {
        if (v.x != 0.0f || v.y != 0.0f || v.w != 0.0f) red_add_v4(a.g_cov2d + 4 * id, v);
      } else {
        if (v.x != 0.0f) atomicAdd(a.g_cov2d + 4 * id, v.x);
        if (v.y != 0.0f) {
          atomicAdd(a.g_cov2d + 4 * id + 1, v.y);
          atomicAdd(a.g_cov2d + 4 * id + 2, v.y);
        }
        if (v.w != 0.0f) atomicAdd(a.g_cov2d + 4 * id + 3, v.w);
      }
    } else if (c == 2) {
      const float v = rec[5];
      rec[5] = 0.0f;
      if (v != 0.0f) atomicAdd(a.g_alpha + id, v);
    } else {
      const int e = c - 3, ch = e / NCH, k = 4 * (e - ch * NCH);
      float4 *src = reinterpret_cast<float4 *>(rec + kShOff + ch * Grad<C>::CSTR + k);
      const float4 v = *src;
      if (v.x == 0.0f && v.y == 0.0f && v.z == 0.0f && v.w == 0.0f) continue;
      *src = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      float *dst = ctx.g_sh + ((id - ctx.item_lo) * 3 + ch) * ctx.sh_stride + k;
      if (k + 4 <= CC && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
        red_add_v4(dst, v);
      } else {
        const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (k + q < CC && vv[q] != 0.0f) atomicAdd(dst + q, vv[q]);
      }
    }
  }
}

// RGB: as in the forward; the gradient staged for the C = 1 reduction is
// then dL/drgb itself (the constant basis makes the product a plain sum).
template <int C, int MAXT, bool BATCHED, bool RGB = false, bool PERSIST = false>
__global__ void __launch_bounds__(MAXT, 1024 / MAXT * 3 / 4 > 0 ? 768 / MAXT : 1)
    raster_backward_kernel(const RasterArgs a) {
  constexpr int CC = Sh<C>::CC, CCP = Sh<C>::CCP, GSH = Sh<C>::GSH;
  constexpr int NV = Grad<C>::NV;  // gm0 gm1 gc0 gc12 gc3 galpha gsh
  extern __shared__ float4 smem4[];
  __shared__ int s_wcount[32];
  __shared__ uint64_t s_bar;  // bulk-copy barrier of the SH rows
  __shared__ int s_work;
  float *smem = reinterpret_cast<float *>(smem4);
  const int B = a.batch;
  const int nthr = blockDim.x, nwarps = nthr >> 5;
  SmemLayout L = carve<C>(smem, B);
  float *s_grad = L.sh + B * GSH;                                         // [B][NV]
  float *s_w = s_grad + B * NV;                                           // [nwarps][16][kWStride]
  float *s_y = s_w + nwarps * 16 * kWStride;                              // [nwarps][16][kYStride]
  int *s_slots = reinterpret_cast<int *>(s_y + nwarps * 16 * kYStride);  // [nwarps][8]
  int *s_touched = s_slots + nwarps * 8;                                  // [B]
  int *wl = s_touched + B + (threadIdx.x >> 5) * B;                       // [nwarps][B]

  if (PERSIST && threadIdx.x == 0) mbar_init(&s_bar);  // once per CTA, before any tile's first wait
  // bulk-copy phases completed by this CTA: the barrier's parity across the
  // tiles of a persistent grid (one tile per CTA: the batch index's parity)
  uint32_t nphase = 0;
  // one tile; false when the CTA must stop (a bulk-copy wait gave up)
  auto run_tile = [&](int64_t work) -> bool {
    const ViewCtx ctx = make_ctx<BATCHED>(a, work);
    if (ctx.gtile < 0) return true;  // CTA-uniform: not a tile of the grid
    if (!PERSIST && threadIdx.x == 0 && sh_bulk_ok<C>(ctx.sh, ctx.sh_stride))
      mbar_init(&s_bar);  // ordered before use by the batch loop's first barrier
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    int gx, gy;
    pixel_of(ctx, t, gx, gy);
    const bool inside = t < ctx.tile_w * ctx.tile_h && gx < ctx.width && gy < ctx.height;
    const int s0 = a.start[ctx.gtile];
    const int n = tile_list_length(a, ctx.gtile, s0);
    if (n <= 0) return true;
    const float px = fmaf((float)gx, ctx.psx, ctx.topleft[0]);
    const float py = fmaf((float)gy, ctx.psy, ctx.topleft[1]);
    float2 Y2[Sh<C>::NY2];
    float *Ws = s_w + warp * 16 * kWStride;
    float *Ys = s_y + warp * 16 * kYStride;
    int *slots = s_slots + warp * 8;
    {
      float Y[CC];
      if constexpr (RGB) Y[0] = 1.0f;
      else sh_basis<C>(ctx.c2w, px, py, Y);
      pack_basis<C>(Y, Y2);
#pragma unroll
      for (int k = 0; k < 16; ++k) Ys[k * kYStride + lane] = k < CC ? Y[k < CC ? k : 0] : 0.0f;
    }
    float fin[3] = {0.0f, 0.0f, 0.0f}, go[3] = {0.0f, 0.0f, 0.0f};
    if (inside) {
      const int64_t pix = 3 * ((int64_t)gy * ctx.width + gx);
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) {
        fin[ch] = ctx.final_img[pix + ch];
        go[ch] = ctx.grad_out[pix + ch];
      }
    }
    float o[3] = {0.0f, 0.0f, 0.0f};
    float T = 1.0f;
    const float thr = a.T_thresh;
    bool done = !inside;
    float tx0, tx1, ty0, ty1;
    tile_bounds(ctx, tx0, tx1, ty0, ty1);
    const float4 blk = warp_block(px, py);

    // zero once; the fold puts each record it reads back to zero
    for (int f = t; f < B * NV; f += nthr) s_grad[f] = 0.0f;
    for (int base = 0; base < n; base += B) {
      if (__syncthreads_and(done)) break;
      const int nb = min(B, n - base);
      for (int j = t; j < nb; j += nthr) s_touched[j] = 0;
      const int nk = load_batch<C, true>(a, ctx, L, s0 + base, nb, t, nthr, tx0, tx1, ty0, ty1,
                                         s_wcount, &s_bar, PERSIST ? (nphase & 1u) : ((uint32_t)(base / B) & 1u));
      if (nk < 0) return false;  // flagged in g_raster_flags
      if (PERSIST && sh_bulk_ok<C>(ctx.sh, ctx.sh_stride)) ++nphase;
      const int nw = __all_sync(kFull, done) ? 0 : warp_list(L, nk, blk, wl, lane);

      int nslot = 0;  // warp-uniform: Gaussians staged in this warp's weight matrix
      for (int j = 0; j < nw; ++j) {
        const int i = wl[j];
        if (__all_sync(kFull, done)) break;
        bool contrib = false;
        float sc[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        float w[3] = {0.0f, 0.0f, 0.0f};
        if (!done) {
          if (T < thr) {
            done = true;
          } else {
            const float al = L.alpha[i];
            const float4 cv = L.cov[i];
            const float2 m = L.mean[i];
            const float2 h = L.box[i];
            const float x = px - m.x, yy = py - m.y;
            const bool outside = fabsf(x) > h.x || fabsf(yy) > h.y;
            const float radial = outside ? 0.0f : radial_of(cv, x, yy);
            if (!outside && !surely_skipped(radial, al)) {
              const float G = gsx_expf_nonpos(-0.5f * radial);
              if (!(al * G < kMinRenderAlpha)) {
                contrib = true;
                float coeff = al * T * G;
                if (isnan(coeff)) coeff = 0.0f;
                const float *s = L.sh + i * GSH;
                float y[3];
#pragma unroll
                for (int ch = 0; ch < 3; ++ch) {
                  y[ch] = RGB ? fmaxf(s[ch * CCP], 0.0f)
                              : fmaxf(fast_sigmoid(sh_logit<C>(s + ch * CCP, Y2)), 0.0f);  // NaN -> 0
                  o[ch] = fmaf(coeff, y[ch], o[ch]);
                }
#pragma unroll
                for (int ch = 0; ch < 3; ++ch)
                  w[ch] = RGB ? coeff * go[ch] : coeff * (y[ch] * (1.0f - y[ch])) * go[ch];
                const float one_m = fmaf(-al, G, 1.0f);
                float inv_one_m;  // gradient path only: the hardware reciprocal (1 ulp)
                asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv_one_m) : "f"(one_m));
                float P = 0.0f;
#pragma unroll
                for (int ch = 0; ch < 3; ++ch) {
                  const float q = (fin[ch] - o[ch]) * inv_one_m;
                  P = fmaf(go[ch], fmaf(y[ch], T, -q), P);
                }
                const float dg = P * al * G;
                const float inv_det = L.inv_det[i];
                const float tmpx = fmaf(x, cv.w, -(yy * cv.z)) * inv_det;
                const float tmpy = fmaf(-x, cv.y, yy * cv.x) * inv_det;
                const float dx = dg * tmpx, dy = dg * tmpy;
                sc[0] = dx;
                sc[1] = dy;
                sc[2] = 0.5f * (dx * tmpx);
                sc[3] = 0.5f * (dx * tmpy);
                sc[4] = 0.5f * (dy * tmpy);
                sc[5] = P * G;
                T = T * one_m;
              }
            }
          }
        }
        if (__ballot_sync(kFull, contrib)) {
          const float r = warp_sum6(sc, lane);
          if ((lane & 3) == 0 && (lane >> 2) < 6 && r != 0.0f)
            atomicAdd(&s_grad[i * NV + (lane >> 2)], r);
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) Ws[(3 * nslot + ch) * kWStride + lane] = w[ch];
          if (lane == 0) {
            slots[nslot] = i;
            s_touched[i] = 1;
          }
          if (++nslot == kSlots) {
            __syncwarp();
            flush_sh_group<C>(Ws, Ys, slots, nslot, s_grad, lane);
            __syncwarp();
            nslot = 0;
          }
        }
      }
      if (nslot > 0) {
        __syncwarp();
        flush_sh_group<C>(Ws, Ys, slots, nslot, s_grad, lane);
        __syncwarp();
      }
      if (!done && T < thr) done = true;
      __syncthreads();
      fold_batch_grads<C>(a, ctx, L, s_grad, s_touched, nk, t, nthr);
    }
    return true;
  };
  if constexpr (PERSIST) {
    for (int64_t work = claim_work<true>(a, &s_work, true); work >= 0;
         work = claim_work<true>(a, &s_work, false))
      if (!run_tile(work)) return;
  } else {
    run_tile(blockIdx.x);
  }
}

// ---- backward with two pixels per thread -----------------------------------
// The same per-pair arithmetic as raster_backward_kernel, with each warp
// covering an 8x8 block of pixels: lane l owns pixel A = (l & 7, l >> 3) and
// pixel B = A + (0, 4) of its warp's block, so one (warp, Gaussian) entry of
// the per-warp lists covers 64 pixels.  On the headline scene this cuts the
// entries that reach the reductions from 3.2 M to 1.9 M while the pixel
// evaluations grow by 5 %: the record loads, the SH row loads, the six-scalar
// butterfly, the weight staging and the shared-memory folds are paid once for
// both pixels.  The decision path (radial, exponential, 1/255, T) stays exact
// and per pixel; the colour and gradient terms of the two pixels run as
// paired float2 operations.
//
// SH gradients: sum_p w_ch(p) Y_k(p) over the warp's 64 pixels as one
// m16n8k16 tensor-core product per group of five Gaussians, in FP16 with a
// high/low split of both operands (hi*hi + hi*lo + lo*hi, FP32 accumulation:
// about 2^-21 relative per product; a weight below 2^-24 is lost, far below
// the gradient tolerance).  Both operands are staged as half2 pairs
// (pixel A, pixel B) of one lane, so a 32-bit word holds the two adjacent
// k values a fragment register wants; rows are 32 words with the column
// XOR-swizzled by (row & 7) << 2, which makes the fragment reads and the
// per-lane writes free of bank conflicts without padding.  The basis is split
// once per warp; the weights once per Gaussian.
constexpr int kP2Cols = 32;  // half2 columns per staged row: 64 pixels

__device__ __forceinline__ int p2_idx(int row, int col) {
  return row * kP2Cols + (col ^ ((row & 7) << 2));
}

__device__ __forceinline__ void split_half2(float a, float b, uint32_t &hi, uint32_t &lo) {
  const __half2 h = __floats2half2_rn(a, b);
  const __half2 l = __floats2half2_rn(a - __low2float(h), b - __high2float(h));
  hi = *reinterpret_cast<const uint32_t *>(&h);
  lo = *reinterpret_cast<const uint32_t *>(&l);
}

__device__ __forceinline__ void mma_f16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                        uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Staging of one warp: weights W[16 rows][64 px] and basis Y[16 k][64 px],
// each as high and low half2 words.
struct P2Stage {
  uint32_t *wh, *wl, *yh, *yl;
};
constexpr int kP2StageWords = 4 * 16 * kP2Cols;

// SH gradients of the staged Gaussians, D[r][k] = sum_p W[r][p] Y[p][k] for
// rows r = 3*slot + channel, added into the batch accumulators.
template <int C>
__device__ __forceinline__ void flush_sh_group2(const P2Stage &S, const int *slots, int nslot,
                                                float *s_grad, int lane) {
  constexpr int CC = Sh<C>::CC;
  constexpr int NT = (CC + 7) / 8;
  constexpr int NV = Grad<C>::NV, CSTR = Grad<C>::CSTR;
  const int g = lane >> 2, tq = lane & 3;
  // hi*hi and the two cross products in separate accumulators: four short
  // dependency chains per flush instead of one of twelve tensor-core latencies
  float d[NT][4], dc[NT][4];
#pragma unroll
  for (int nt = 0; nt < NT; ++nt)
#pragma unroll
    for (int e = 0; e < 4; ++e) d[nt][e] = dc[nt][e] = 0.0f;
#pragma unroll
  for (int ks = 0; ks < 4; ++ks) {
    const int c0 = 8 * ks + tq, c1 = c0 + 4;
    const uint32_t ah[4] = {S.wh[p2_idx(g, c0)], S.wh[p2_idx(g + 8, c0)], S.wh[p2_idx(g, c1)],
                            S.wh[p2_idx(g + 8, c1)]};
    const uint32_t al[4] = {S.wl[p2_idx(g, c0)], S.wl[p2_idx(g + 8, c0)], S.wl[p2_idx(g, c1)],
                            S.wl[p2_idx(g + 8, c1)]};
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
      const int n = 8 * nt + g;
      const uint32_t bh0 = S.yh[p2_idx(n, c0)], bh1 = S.yh[p2_idx(n, c1)];
      const uint32_t bl0 = S.yl[p2_idx(n, c0)], bl1 = S.yl[p2_idx(n, c1)];
      mma_f16(d[nt], ah, bh0, bh1);
      mma_f16(dc[nt], ah, bl0, bl1);
      mma_f16(dc[nt], al, bh0, bh1);
    }
  }
  // this lane's two rows: r = g and g + 8, i.e. (slot, channel) pairs
  const int rows = 3 * nslot;
  const int sl0 = g / 3, sl1 = (g + 8) / 3;
  const int base0 = g < rows ? slots[sl0] * NV + kShOff + (g - 3 * sl0) * CSTR : -1;
  const int base1 = g + 8 < rows ? slots[sl1] * NV + kShOff + (g + 8 - 3 * sl1) * CSTR : -1;
#pragma unroll
  for (int nt = 0; nt < NT; ++nt)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int base = (e & 2) ? base1 : base0;
      const int k = 8 * nt + 2 * tq + (e & 1);
      const float v = d[nt][e] + dc[nt][e];
      if (base >= 0 && k < CC && v != 0.0f) atomicAdd(&s_grad[base + k], v);
    }
}

// Pixels of thread t: 8x8 warp blocks over the tile (tile_w and tile_h
// multiples of 8); pixel B lies four rows below pixel A.
__device__ __forceinline__ void pixel_of2(const ViewCtx &c, int t, int &gx, int &gy) {
  const int w = t >> 5, l = t & 31, bpr = c.tile_w >> 3;
  gx = (c.tile % c.n_tiles_w) * c.tile_w + (w % bpr) * 8 + (l & 7);
  gy = (c.tile / c.n_tiles_w) * c.tile_h + (w / bpr) * 8 + (l >> 3);
}

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// Bounds of the pixel centres of this warp's 8x8 block (both pixels of every
// lane).
__device__ __forceinline__ float4 warp_block2(float px, float py0, float py1) {
  float x0 = px, x1 = px, y0 = fminf(py0, py1), y1 = fmaxf(py0, py1);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    x0 = fminf(x0, __shfl_xor_sync(kFull, x0, o));
    x1 = fmaxf(x1, __shfl_xor_sync(kFull, x1, o));
    y0 = fminf(y0, __shfl_xor_sync(kFull, y0, o));
    y1 = fmaxf(y1, __shfl_xor_sync(kFull, y1, o));
  }
  return make_float4(x0, x1, y0, y1);
}

template <int C, int MAXT, bool BATCHED, bool RGB = false, bool PERSIST = false>
__global__ void __launch_bounds__(MAXT, MAXT <= 128 ? 4 : 512 / MAXT)
    raster_backward2_kernel(const RasterArgs a) {
  constexpr int CC = Sh<C>::CC, CCP = Sh<C>::CCP, GSH = Sh<C>::GSH;
  constexpr int NV = Grad<C>::NV;
  extern __shared__ float4 smem4[];
  __shared__ int s_wcount[32];
  __shared__ uint64_t s_bar;  // bulk-copy barrier of the SH rows
  __shared__ int s_work;
  float *smem = reinterpret_cast<float *>(smem4);
  const int B = a.batch;
  const int nthr = blockDim.x, nwarps = nthr >> 5;
  SmemLayout L = carve<C>(smem, B);
  float *s_grad = L.sh + B * GSH;                                              // [B][NV]
  uint32_t *s_stage = reinterpret_cast<uint32_t *>(s_grad + B * NV);          // [nwarps][4][16][32]
  int *s_slots = reinterpret_cast<int *>(s_stage + nwarps * kP2StageWords);  // [nwarps][8]
  int *s_touched = s_slots + nwarps * 8;                                       // [B]
  int *wl = s_touched + B + (threadIdx.x >> 5) * B;                            // [nwarps][B]

  if (PERSIST && threadIdx.x == 0) mbar_init(&s_bar);  // once per CTA, before any tile's first wait
  // bulk-copy phases completed by this CTA: the barrier's parity across the
  // tiles of a persistent grid (one tile per CTA: the batch index's parity)
  uint32_t nphase = 0;
  // one tile; false when the CTA must stop (a bulk-copy wait gave up)
  auto run_tile = [&](int64_t work) -> bool {
    const ViewCtx ctx = make_ctx<BATCHED>(a, work);
    if (ctx.gtile < 0) return true;  // CTA-uniform: not a tile of the grid
    if (!PERSIST && threadIdx.x == 0 && sh_bulk_ok<C>(ctx.sh, ctx.sh_stride))
      mbar_init(&s_bar);  // ordered before use by the batch loop's first barrier
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    int gx, gy0;
    pixel_of2(ctx, t, gx, gy0);
    const int gy1 = gy0 + 4;
    const bool in0 = gx < ctx.width && gy0 < ctx.height;
    const bool in1 = gx < ctx.width && gy1 < ctx.height;
    const int s0 = a.start[ctx.gtile];
    const int n = tile_list_length(a, ctx.gtile, s0);
    if (n <= 0) return true;
    const float px = fmaf((float)gx, ctx.psx, ctx.topleft[0]);
    const float py0 = fmaf((float)gy0, ctx.psy, ctx.topleft[1]);
    const float py1 = fmaf((float)gy1, ctx.psy, ctx.topleft[1]);
    P2Stage S;
    S.wh = s_stage + warp * kP2StageWords;
    S.wl = S.wh + 16 * kP2Cols;
    S.yh = S.wl + 16 * kP2Cols;
    S.yl = S.yh + 16 * kP2Cols;
    int *slots = s_slots + warp * 8;
    float2 Y2a[Sh<C>::NY2], Y2b[Sh<C>::NY2];
    {
      float Ya[CC], Yb[CC];
      if constexpr (RGB) {
        Ya[0] = 1.0f;
        Yb[0] = 1.0f;
      } else {
        sh_basis<C>(ctx.c2w, px, py0, Ya);
        sh_basis<C>(ctx.c2w, px, py1, Yb);
      }
      pack_basis<C>(Ya, Y2a);
      pack_basis<C>(Yb, Y2b);
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        uint32_t hi = 0u, lo = 0u;
        if (k < CC) split_half2(Ya[k < CC ? k : 0], Yb[k < CC ? k : 0], hi, lo);
        S.yh[p2_idx(k, lane)] = hi;
        S.yl[p2_idx(k, lane)] = lo;
        S.wh[p2_idx(k, lane)] = 0u;  // rows never staged stay finite
        S.wl[p2_idx(k, lane)] = 0u;
      }
    }
    // per-pixel state as (pixel A, pixel B) pairs
    float2 fin2[3] = {f2(0.0f, 0.0f), f2(0.0f, 0.0f), f2(0.0f, 0.0f)};
    float2 go2[3] = {f2(0.0f, 0.0f), f2(0.0f, 0.0f), f2(0.0f, 0.0f)};
    if (in0) {
      const int64_t pix = 3 * ((int64_t)gy0 * ctx.width + gx);
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) {
        fin2[ch].x = ctx.final_img[pix + ch];
        go2[ch].x = ctx.grad_out[pix + ch];
      }
    }
    if (in1) {
      const int64_t pix = 3 * ((int64_t)gy1 * ctx.width + gx);
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) {
        fin2[ch].y = ctx.final_img[pix + ch];
        go2[ch].y = ctx.grad_out[pix + ch];
      }
    }
    float2 o[3] = {f2(0.0f, 0.0f), f2(0.0f, 0.0f), f2(0.0f, 0.0f)};
    float2 T2 = f2(1.0f, 1.0f);
    const float thr = a.T_thresh;
    bool done0 = !in0, done1 = !in1;
    float tx0, tx1, ty0, ty1;
    tile_bounds(ctx, tx0, tx1, ty0, ty1);
    const float4 blk = warp_block2(px, py0, py1);

    // the accumulators start at zero; the fold puts each record it reads
    // back to zero, and untouched records are never written
    for (int f = t; f < B * NV; f += nthr) s_grad[f] = 0.0f;
    for (int base = 0; base < n; base += B) {
      if (__syncthreads_and(done0 && done1)) break;
      const int nb = min(B, n - base);
      for (int j = t; j < nb; j += nthr) s_touched[j] = 0;
      const int nk = load_batch<C, true>(a, ctx, L, s0 + base, nb, t, nthr, tx0, tx1, ty0, ty1,
                                         s_wcount, &s_bar, PERSIST ? (nphase & 1u) : ((uint32_t)(base / B) & 1u));
      if (nk < 0) return false;  // flagged in g_raster_flags
      if (PERSIST && sh_bulk_ok<C>(ctx.sh, ctx.sh_stride)) ++nphase;
      const int nw = __all_sync(kFull, done0 && done1) ? 0 : warp_list(L, nk, blk, wl, lane);

      int nslot = 0;  // warp-uniform: Gaussians staged in this warp's weight matrix
      for (int j = 0; j < nw; ++j) {
        const int i = wl[j];
        if (__all_sync(kFull, done0 && done1)) break;
        // a pixel stops before the Gaussian once its transmittance is below the
        // threshold (the reference's per-Gaussian test)
        if (!done0 && T2.x < thr) done0 = true;
        if (!done1 && T2.y < thr) done1 = true;
        bool c0 = false, c1 = false;
        float G0 = 0.0f, G1 = 0.0f, tx_0 = 0.0f, ty_0 = 0.0f, tx_1 = 0.0f, ty_1 = 0.0f;
        const float al = L.alpha[i];
        const float4 cv = L.cov[i];
        const float2 m = L.mean[i];
        if (!(done0 && done1)) {
          // both pixels' decision paths side by side, without branches: the
          // radial of gs/src/include/kernels.h:172-187 (one det per Gaussian,
          // IEEE division), then the exact exponential.  The two pixels share
          // x (same column); every other step runs as a paired float2
          // operation, each half rounded as its scalar form (-(y*z) ==
          // y*(-z) and a - b == a + (-b) exactly).
          const float2 h = L.box[i];
          const float x = px - m.x;
          const float2 y = __fadd2_rn(f2(py0, py1), f2(-m.y, -m.y));
          const float2 X = f2(x, x);
          const float det = fmaf(cv.x, cv.w, -(cv.y * cv.z));
          const float2 txp = __ffma2_rn(X, f2(cv.w, cv.w), __fmul2_rn(y, f2(-cv.z, -cv.z)));
          const float2 typ = __ffma2_rn(f2(-x, -x), f2(cv.y, cv.y), __fmul2_rn(y, f2(cv.x, cv.x)));
          tx_0 = txp.x;
          tx_1 = txp.y;
          ty_0 = typ.x;
          ty_1 = typ.y;
          const float2 num = __ffma2_rn(txp, X, __fmul2_rn(typ, y));
          float r0 = num.x / det;
          float r1 = num.y / det;
          if (r0 < 0.0f) r0 = 1000.0f;
          if (r1 < 0.0f) r1 = 1000.0f;
          const bool xin = !(fabsf(x) > h.x);
          const bool live0 = !done0 && xin && !(fabsf(y.x) > h.y) && !surely_skipped(r0, al);
          const bool live1 = !done1 && xin && !(fabsf(y.y) > h.y) && !surely_skipped(r1, al);
          const float2 e = gsx_expf_nonpos2(__fmul2_rn(f2(-0.5f, -0.5f), f2(r0, r1)));
          const float2 ae = __fmul2_rn(f2(al, al), e);
          c0 = live0 && !(ae.x < kMinRenderAlpha);
          c1 = live1 && !(ae.y < kMinRenderAlpha);
          G0 = c0 ? e.x : 0.0f;
          G1 = c1 ? e.y : 0.0f;
        }
        float sc[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        float2 w[3] = {f2(0.0f, 0.0f), f2(0.0f, 0.0f), f2(0.0f, 0.0f)};
        if (c0 || c1) {
          // both pixels at once; a pixel that does not take this Gaussian has
          // G = 0, so its colour sums and weights are unchanged / zero (its
          // other terms are finite whenever the Gaussian's record is)
          const float2 Gp = f2(G0, G1);
          const float2 al2 = f2(al, al);
          float2 coeff = __fmul2_rn(__fmul2_rn(al2, T2), Gp);
          if (isnan(coeff.x)) coeff.x = 0.0f;
          if (isnan(coeff.y)) coeff.y = 0.0f;
          const float *s = L.sh + i * GSH;
          float2 yv[3];
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) {
            if constexpr (RGB) {
              const float v = fmaxf(s[ch * CCP], 0.0f);
              yv[ch] = f2(v, v);
            } else {
              yv[ch] = f2(fmaxf(fast_sigmoid(sh_logit<C>(s + ch * CCP, Y2a)), 0.0f),  // NaN -> 0
                          fmaxf(fast_sigmoid(sh_logit<C>(s + ch * CCP, Y2b)), 0.0f));
            }
            o[ch] = __ffma2_rn(coeff, yv[ch], o[ch]);
          }
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) {
            if constexpr (RGB) {
              w[ch] = __fmul2_rn(coeff, go2[ch]);
            } else {
              // y (1 - y), with 1 - y as fma(y, -1, 1)
              const float2 yy = __fmul2_rn(yv[ch], __ffma2_rn(yv[ch], f2(-1.0f, -1.0f), f2(1.0f, 1.0f)));
              w[ch] = __fmul2_rn(__fmul2_rn(coeff, yy), go2[ch]);
            }
          }
          const float2 one_m = __ffma2_rn(f2(-al, -al), Gp, f2(1.0f, 1.0f));
          float inv0, inv1;  // gradient path only: the hardware reciprocal (1 ulp)
          asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv0) : "f"(one_m.x));
          asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv1) : "f"(one_m.y));
          const float2 inv_one_m = f2(inv0, inv1);
          float2 P = f2(0.0f, 0.0f);
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) {
            // -q = (out - final) / (1 - aG): o - fin as fma(fin, -1, o), exact
            const float2 nq = __fmul2_rn(__ffma2_rn(fin2[ch], f2(-1.0f, -1.0f), o[ch]), inv_one_m);
            P = __ffma2_rn(go2[ch], __ffma2_rn(yv[ch], T2, nq), P);
          }
          const float2 dg = __fmul2_rn(__fmul2_rn(P, al2), Gp);
          const float inv_det = L.inv_det[i];
          const float2 idet = f2(inv_det, inv_det);
          const float2 tmpx = __fmul2_rn(f2(tx_0, tx_1), idet);
          const float2 tmpy = __fmul2_rn(f2(ty_0, ty_1), idet);
          const float2 dx = __fmul2_rn(dg, tmpx), dy = __fmul2_rn(dg, tmpy);
          const float2 s2 = __fmul2_rn(f2(0.5f, 0.5f), __fmul2_rn(dx, tmpx));
          const float2 s3 = __fmul2_rn(f2(0.5f, 0.5f), __fmul2_rn(dx, tmpy));
          const float2 s4 = __fmul2_rn(f2(0.5f, 0.5f), __fmul2_rn(dy, tmpy));
          const float2 s5 = __fmul2_rn(P, Gp);
          sc[0] = dx.x + dx.y;
          sc[1] = dy.x + dy.y;
          sc[2] = s2.x + s2.y;
          sc[3] = s3.x + s3.y;
          sc[4] = s4.x + s4.y;
          sc[5] = s5.x + s5.y;
          if (c0) T2.x = T2.x * one_m.x;
          if (c1) T2.y = T2.y * one_m.y;
        }
        if (__ballot_sync(kFull, c0 || c1)) {
          const float r = warp_sum6(sc, lane);
          if ((lane & 3) == 0 && (lane >> 2) < 6 && r != 0.0f)
            atomicAdd(&s_grad[i * NV + (lane >> 2)], r);
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) {
            uint32_t hi, lo;
            split_half2(w[ch].x, w[ch].y, hi, lo);
            S.wh[p2_idx(3 * nslot + ch, lane)] = hi;
            S.wl[p2_idx(3 * nslot + ch, lane)] = lo;
          }
          if (lane == 0) {
            slots[nslot] = i;
            s_touched[i] = 1;
          }
          if (++nslot == kSlots) {
            __syncwarp();
            flush_sh_group2<C>(S, slots, nslot, s_grad, lane);
            __syncwarp();
            nslot = 0;
          }
        }
      }
      if (nslot > 0) {
        __syncwarp();
        flush_sh_group2<C>(S, slots, nslot, s_grad, lane);
        __syncwarp();
      }
      if (!done0 && T2.x < thr) done0 = true;
      if (!done1 && T2.y < thr) done1 = true;
      __syncthreads();
      fold_batch_grads<C>(a, ctx, L, s_grad, s_touched, nk, t, nthr);
    }
    return true;
  };
  if constexpr (PERSIST) {
    for (int64_t work = claim_work<true>(a, &s_work, true); work >= 0;
         work = claim_work<true>(a, &s_work, false))
      if (!run_tile(work)) return;
  } else {
    run_tile(blockIdx.x);
  }
}

// Forward with two pixels per thread over 8x8 warp blocks (the layout of
// raster_backward2_kernel): the record and SH row loads of an entry serve
// both pixels, and the two pixels' exact decision paths run side by side
// without branches.  Same arithmetic per pair as raster_forward_kernel.
template <int C, int MAXT, bool BATCHED, bool RGB = false, bool PERSIST = false>
__global__ void __launch_bounds__(MAXT, MAXT <= 128 ? 5 : 640 / MAXT)
    raster_forward2_kernel(const RasterArgs a) {
  constexpr int GSH = Sh<C>::GSH, CCP = Sh<C>::CCP;
  extern __shared__ float4 smem4[];
  __shared__ int s_wcount[32];
  __shared__ uint64_t s_bar;  // bulk-copy barrier of the SH rows
  __shared__ int s_work;
  const int nthr = blockDim.x;
  const int B = a.batch;
  SmemLayout L = carve<C>(reinterpret_cast<float *>(smem4), B);
  int *wl = reinterpret_cast<int *>(L.sh + B * GSH) + (threadIdx.x >> 5) * B;  // [nwarps][B]

  if (PERSIST && threadIdx.x == 0) mbar_init(&s_bar);  // once per CTA, before any tile's first wait
  // bulk-copy phases completed by this CTA: the barrier's parity across the
  // tiles of a persistent grid (one tile per CTA: the batch index's parity)
  uint32_t nphase = 0;
  // one tile; false when the CTA must stop (a bulk-copy wait gave up)
  auto run_tile = [&](int64_t work) -> bool {
    const ViewCtx ctx = make_ctx<BATCHED>(a, work);
    if (ctx.gtile < 0) return true;  // CTA-uniform: not a tile of the grid
    if (!PERSIST && threadIdx.x == 0 && sh_bulk_ok<C>(ctx.sh, ctx.sh_stride))
      mbar_init(&s_bar);  // ordered before use by the batch loop's first barrier
    const int t = threadIdx.x, lane = t & 31;
    int gx, gy0;
    pixel_of2(ctx, t, gx, gy0);
    const int gy1 = gy0 + 4;
    const bool in0 = gx < ctx.width && gy0 < ctx.height;
    const bool in1 = gx < ctx.width && gy1 < ctx.height;
    const int s0 = a.start[ctx.gtile];
    const int n = tile_list_length(a, ctx.gtile, s0);
    if (n <= 0) {
      if (ctx.write_empty) {
        if (in0) {
          float *dst = ctx.out + 3 * ((int64_t)gy0 * ctx.width + gx);
          dst[0] = dst[1] = dst[2] = 0.0f;
        }
        if (in1) {
          float *dst = ctx.out + 3 * ((int64_t)gy1 * ctx.width + gx);
          dst[0] = dst[1] = dst[2] = 0.0f;
        }
      }
      return true;
    }
    const float px = fmaf((float)gx, ctx.psx, ctx.topleft[0]);
    const float py0 = fmaf((float)gy0, ctx.psy, ctx.topleft[1]);
    const float py1 = fmaf((float)gy1, ctx.psy, ctx.topleft[1]);
    float2 Y2a[Sh<C>::NY2], Y2b[Sh<C>::NY2];
    {
      float Ya[Sh<C>::CC], Yb[Sh<C>::CC];
      if constexpr (RGB) {
        Ya[0] = 1.0f;
        Yb[0] = 1.0f;
      } else {
        sh_basis<C>(ctx.c2w, px, py0, Ya);
        sh_basis<C>(ctx.c2w, px, py1, Yb);
      }
      pack_basis<C>(Ya, Y2a);
      pack_basis<C>(Yb, Y2b);
    }
    float2 o[3] = {f2(0.0f, 0.0f), f2(0.0f, 0.0f), f2(0.0f, 0.0f)};
    float2 T2 = f2(1.0f, 1.0f);
    const float thr = a.T_thresh;
    bool done0 = !in0, done1 = !in1;
    float tx0, tx1, ty0, ty1;
    tile_bounds(ctx, tx0, tx1, ty0, ty1);
    const float4 blk = warp_block2(px, py0, py1);

    for (int base = 0; base < n; base += B) {
      if (__syncthreads_and(done0 && done1)) break;
      const int nb = min(B, n - base);
      const int nk = load_batch<C, false>(a, ctx, L, s0 + base, nb, t, nthr, tx0, tx1, ty0, ty1,
                                          s_wcount, &s_bar, PERSIST ? (nphase & 1u) : ((uint32_t)(base / B) & 1u));
      if (nk < 0) return false;  // flagged in g_raster_flags
      if (PERSIST && sh_bulk_ok<C>(ctx.sh, ctx.sh_stride)) ++nphase;
      const int nw = __all_sync(kFull, done0 && done1) ? 0 : warp_list(L, nk, blk, wl, lane);
      for (int j = 0; j < nw; ++j) {
        if (!done0 && T2.x < thr) done0 = true;
        if (!done1 && T2.y < thr) done1 = true;
        if (__all_sync(kFull, done0 && done1)) break;
        if (done0 && done1) continue;
        const int i = wl[j];
        const float al = L.alpha[i];
        const float4 cv = L.cov[i];
        const float2 m = L.mean[i];
        const float2 h = L.box[i];
        // paired float2 steps, each half rounded as in the one-pixel kernel
        const float x = px - m.x;
        const float2 y = __fadd2_rn(f2(py0, py1), f2(-m.y, -m.y));
        const float2 X = f2(x, x);
        const float det = fmaf(cv.x, cv.w, -(cv.y * cv.z));
        const float2 txp = __ffma2_rn(X, f2(cv.w, cv.w), __fmul2_rn(y, f2(-cv.z, -cv.z)));
        const float2 typ = __ffma2_rn(f2(-x, -x), f2(cv.y, cv.y), __fmul2_rn(y, f2(cv.x, cv.x)));
        const float2 num = __ffma2_rn(txp, X, __fmul2_rn(typ, y));
        float r0 = num.x / det;
        float r1 = num.y / det;
        if (r0 < 0.0f) r0 = 1000.0f;
        if (r1 < 0.0f) r1 = 1000.0f;
        const bool xin = !(fabsf(x) > h.x);
        const bool live0 = !done0 && xin && !(fabsf(y.x) > h.y) && !surely_skipped(r0, al);
        const bool live1 = !done1 && xin && !(fabsf(y.y) > h.y) && !surely_skipped(r1, al);
        const float2 e = gsx_expf_nonpos2(__fmul2_rn(f2(-0.5f, -0.5f), f2(r0, r1)));
        const float2 ae = __fmul2_rn(f2(al, al), e);
        const bool c0 = live0 && !(ae.x < kMinRenderAlpha);
        const bool c1 = live1 && !(ae.y < kMinRenderAlpha);
        if (!(c0 || c1)) continue;
        const float2 Gp = f2(c0 ? e.x : 0.0f, c1 ? e.y : 0.0f);
        float2 coeff = __fmul2_rn(__fmul2_rn(f2(al, al), T2), Gp);
        if (isnan(coeff.x)) coeff.x = 0.0f;
        if (isnan(coeff.y)) coeff.y = 0.0f;
        const float *s = L.sh + i * GSH;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
          float2 y;
          if constexpr (RGB) {
            y = f2(s[ch * CCP], s[ch * CCP]);
          } else {
            y = f2(fast_sigmoid(sh_logit<C>(s + ch * CCP, Y2a)),
                   fast_sigmoid(sh_logit<C>(s + ch * CCP, Y2b)));
          }
          // coeff is finite, so y * coeff is NaN exactly when y is; fmaxf
          // returns its non-NaN operand and y >= 0: the reference's
          // `if isnan(y * coeff) y = 0`
          y = f2(fmaxf(y.x, 0.0f), fmaxf(y.y, 0.0f));
          o[ch] = __ffma2_rn(coeff, y, o[ch]);
        }
        const float2 one_m = __ffma2_rn(f2(-al, -al), Gp, f2(1.0f, 1.0f));
        if (c0) T2.x = T2.x * one_m.x;
        if (c1) T2.y = T2.y * one_m.y;
      }
      if (!done0 && T2.x < thr) done0 = true;
      if (!done1 && T2.y < thr) done1 = true;
    }
    if (in0) {
      float *dst = ctx.out + 3 * ((int64_t)gy0 * ctx.width + gx);
      dst[0] = o[0].x;
      dst[1] = o[1].x;
      dst[2] = o[2].x;
    }
    if (in1) {
      float *dst = ctx.out + 3 * ((int64_t)gy1 * ctx.width + gx);
      dst[0] = o[0].y;
      dst[1] = o[1].y;
      dst[2] = o[2].y;
    }
    return true;
  };
  if constexpr (PERSIST) {
    for (int64_t work = claim_work<true>(a, &s_work, true); work >= 0;
         work = claim_work<true>(a, &s_work, false))
      if (!run_tile(work)) return;
  } else {
    run_tile(blockIdx.x);
  }
}

template <int C>
size_t fwd_smem(int B, int nthr) {
  return (size_t)B * (kRecordFloats + Sh<C>::GSH) * sizeof(float) +
         (size_t)(nthr / 32) * B * sizeof(int);
}

template <int C>
size_t bwd_smem(int B, int nthr) {
  constexpr int NV = Grad<C>::NV;
  const int nwarps = nthr / 32;
  return (size_t)B * (kRecordFloats + Sh<C>::GSH + NV + 1) * sizeof(float) +
         (size_t)nwarps * (16 * kWStride + 16 * kYStride + 8 + B) * sizeof(float);
}

inline int block_threads(const RasterArgs &a) { return (a.tile_w * a.tile_h + 31) / 32 * 32; }

// cudaFuncSetAttribute only when a kernel needs more dynamic shared memory
// than it was last given (it is not a stream operation, but costs host time
// per call).  `done` must be private to one kernel: each launcher
// instantiation below owns its own.
template <typename K>
cudaError_t ensure_smem(K kernel, size_t smem, size_t &done) {
  if (smem <= done) return cudaSuccess;
  cudaError_t e =
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) done = smem;
  return e;
}

// Grid of a raster launch over a.n_work = `items` tiles: one CTA per tile,
// or, with a work counter, as many CTAs as the SMs hold at once (the counter
// is zeroed first, on the launch's stream).
template <typename K>
cudaError_t raster_grid(K kernel, int nthr, size_t smem, int64_t items, RasterArgs &a,
                        cudaStream_t s, unsigned &grid) {
  a.n_work = items;
  grid = (unsigned)items;
  if (!a.work_counter) return cudaSuccess;
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, nthr, smem);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.work_counter, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  const int64_t resident = (int64_t)sms * (per_sm > 0 ? per_sm : 1);
  grid = (unsigned)(items < resident ? items : resident);
  return cudaSuccess;
}

// The two-pixel raster kernels cover tiles made of 8x8 blocks, up to 1024
// pixels.
inline bool two_pixel_tiles(const RasterArgs &a) {
  return a.tile_w % 8 == 0 && a.tile_h % 8 == 0 && a.tile_w * a.tile_h <= 1024;
}

// Pixels per thread of the raster backward: a.pixels_per_thread 1 or 2, or
// 0 for two wherever the tile is made of 8x8 blocks (measured on the 1M-
// Gaussian 1080p view: 1.72 against 1.98 ms).
inline bool use_two_pixels(const RasterArgs &a) {
  return a.pixels_per_thread != 1 && two_pixel_tiles(a);
}

// The forward takes two pixels per thread only when asked for (0 means one:
// its work per list entry is nearly all per pixel, and on the same view the
// two-pixel forward measured 0.729 against 0.719 ms).
inline bool use_two_pixels_fwd(const RasterArgs &a) {
  return a.pixels_per_thread == 2 && two_pixel_tiles(a);
}

// Gaussians per shared-memory batch of the one-pixel forward (44 KB at 160,
// four CTAs per SM).  Measured on the 1080p view (256 threads per 16x16 tile):
// 96 -> 0.703 ms, 128 -> 0.6926, 160 -> 0.6898 (three runs each), 192 -> 0.713.
#ifndef GSX_FWD_BATCH
#define GSX_FWD_BATCH 160
#endif

template <int C, int MAXT, bool BATCHED, bool EXTRAS, bool RGB = false>
int launch_fwd_tt(RasterArgs a, int64_t grid, cudaStream_t s) {
  const int nthr = block_threads(a);
  a.batch = nthr < GSX_FWD_BATCH ? nthr : GSX_FWD_BATCH;
  const size_t smem = fwd_smem<C>(a.batch, nthr);
  static size_t attr_done = 0, attr_done_p = 0;
  cudaError_t e = ensure_smem(raster_forward_kernel<C, MAXT, BATCHED, EXTRAS, RGB>, smem, attr_done);
  if (e != cudaSuccess) return cuda_status(e, "raster_forward smem attribute");
  unsigned launch_grid = 0;
  if constexpr (BATCHED) {
    if (a.work_counter) {  // persistent grid over the batch's tiles
      auto kp = raster_forward_kernel<C, MAXT, BATCHED, EXTRAS, RGB, true>;
      e = ensure_smem(kp, smem, attr_done_p);
      if (e == cudaSuccess) e = raster_grid(kp, nthr, smem, grid, a, s, launch_grid);
      if (e != cudaSuccess) return cuda_status(e, "raster grid");
      count_launches(1);
      kp<<<launch_grid, nthr, smem, s>>>(a);
      return cuda_status(cudaGetLastError(), "raster_forward_kernel launch");
    }
  }
  a.work_counter = nullptr;
  e = raster_grid(raster_forward_kernel<C, MAXT, BATCHED, EXTRAS, RGB>, nthr, smem, grid, a, s, launch_grid);
  if (e != cudaSuccess) return cuda_status(e, "raster grid");
  count_launches(1);
  raster_forward_kernel<C, MAXT, BATCHED, EXTRAS, RGB><<<launch_grid, nthr, smem, s>>>(a);
  return cuda_status(cudaGetLastError(), "raster_forward_kernel launch");
}

template <int C, int MAXT, bool BATCHED, bool RGB = false>
int launch_fwd2_tt(RasterArgs a, int64_t grid, cudaStream_t s) {
  const int nthr = a.tile_w * a.tile_h / 2;
  a.batch = nthr < 128 ? nthr : 128;
  const size_t smem = fwd_smem<C>(a.batch, nthr);
  static size_t attr_done = 0, attr_done_p = 0;
  cudaError_t e = ensure_smem(raster_forward2_kernel<C, MAXT, BATCHED, RGB>, smem, attr_done);
  if (e != cudaSuccess) return cuda_status(e, "raster_forward2 smem attribute");
  unsigned launch_grid = 0;
  if constexpr (BATCHED) {
    if (a.work_counter) {  // persistent grid over the batch's tiles
      auto kp = raster_forward2_kernel<C, MAXT, BATCHED, RGB, true>;
      e = ensure_smem(kp, smem, attr_done_p);
      if (e == cudaSuccess) e = raster_grid(kp, nthr, smem, grid, a, s, launch_grid);
      if (e != cudaSuccess) return cuda_status(e, "raster grid");
      count_launches(1);
      kp<<<launch_grid, nthr, smem, s>>>(a);
      return cuda_status(cudaGetLastError(), "raster_forward2_kernel launch");
    }
  }
  a.work_counter = nullptr;
  e = raster_grid(raster_forward2_kernel<C, MAXT, BATCHED, RGB>, nthr, smem, grid, a, s, launch_grid);
  if (e != cudaSuccess) return cuda_status(e, "raster grid");
  count_launches(1);
  raster_forward2_kernel<C, MAXT, BATCHED, RGB><<<launch_grid, nthr, smem, s>>>(a);
  return cuda_status(cudaGetLastError(), "raster_forward2_kernel launch");
}

template <int C, bool BATCHED, bool RGB = false>
int launch_fwd2_t(const RasterArgs &a, int64_t grid, cudaStream_t s) {
  const int nthr = a.tile_w * a.tile_h / 2;
  return nthr <= 128   ? launch_fwd2_tt<C, 128, BATCHED, RGB>(a, grid, s)
         : nthr <= 256 ? launch_fwd2_tt<C, 256, BATCHED, RGB>(a, grid, s)
                       : launch_fwd2_tt<C, 512, BATCHED, RGB>(a, grid, s);
}

template <int C, bool BATCHED>
int launch_fwd_t(const RasterArgs &a, int64_t grid, cudaStream_t s) {
  if constexpr (!BATCHED) {
    if (a.has_bg || a.alpha_out || a.depth_out)
      return block_threads(a) <= 256 ? launch_fwd_tt<C, 256, false, true>(a, grid, s)
                                     : launch_fwd_tt<C, 1024, false, true>(a, grid, s);
  }
  if (use_two_pixels_fwd(a)) return launch_fwd2_t<C, BATCHED>(a, grid, s);
  return block_threads(a) <= 256 ? launch_fwd_tt<C, 256, BATCHED, false>(a, grid, s)
                                 : launch_fwd_tt<C, 1024, BATCHED, false>(a, grid, s);
}

template <int C, int MAXT, bool BATCHED, bool RGB = false>
int launch_bwd_tt(RasterArgs a, int64_t grid, cudaStream_t s) {
  const int nthr = block_threads(a);
  a.vec_grads = ((reinterpret_cast<uintptr_t>(a.g_mean2d) & 7) == 0 &&
                 (reinterpret_cast<uintptr_t>(a.g_cov2d) & 15) == 0)
                    ? 1
                    : 0;
  a.batch = nthr < 64 ? nthr : 64;
  const size_t smem = bwd_smem<C>(a.batch, nthr);
  static size_t attr_done = 0, attr_done_p = 0;
  cudaError_t e = ensure_smem(raster_backward_kernel<C, MAXT, BATCHED, RGB>, smem, attr_done);
  if (e != cudaSuccess) return cuda_status(e, "raster_backward smem attribute");
  unsigned launch_grid = 0;
  if constexpr (BATCHED) {
    if (a.work_counter) {  // persistent grid over the batch's tiles
      auto kp = raster_backward_kernel<C, MAXT, BATCHED, RGB, true>;
      e = ensure_smem(kp, smem, attr_done_p);
      if (e == cudaSuccess) e = raster_grid(kp, nthr, smem, grid, a, s, launch_grid);
      if (e != cudaSuccess) return cuda_status(e, "raster grid");
      count_launches(1);
      kp<<<launch_grid, nthr, smem, s>>>(a);
      return cuda_status(cudaGetLastError(), "raster_backward_kernel launch");
    }
  }
  a.work_counter = nullptr;
  e = raster_grid(raster_backward_kernel<C, MAXT, BATCHED, RGB>, nthr, smem, grid, a, s, launch_grid);
  if (e != cudaSuccess) return cuda_status(e, "raster grid");
  count_launches(1);
  raster_backward_kernel<C, MAXT, BATCHED, RGB><<<launch_grid, nthr, smem, s>>>(a);
  return cuda_status(cudaGetLastError(), "raster_backward_kernel launch");
}

// Gaussians per shared-memory batch of the two-pixel backward (a multiple of
// 4): with 128 threads per 16x16 tile, 48 is the largest that keeps four CTAs
// per SM (56.5 KB each; 52 needs 58.4 KB).  Measured on the 1080p view: 36 ->
// 1.740 ms, 40 -> 1.717, 44 -> 1.698 with 20-float SH-gradient rows; 44 ->
// 1.673 and 48 -> 1.657 with 16-float rows.
#ifndef GSX_BWD2_BATCH
#define GSX_BWD2_BATCH 48
#endif

template <int C>
size_t bwd2_smem(int B, int nthr) {
  constexpr int NV = Grad<C>::NV;
  const int nwarps = nthr / 32;
  return (size_t)B * (kRecordFloats + Sh<C>::GSH + NV + 1) * sizeof(float) +
         (size_t)nwarps * (kP2StageWords + 8 + B) * sizeof(uint32_t);
}


template <int C, int MAXT, bool BATCHED, bool RGB = false>
int launch_bwd2_tt(RasterArgs a, int64_t grid, cudaStream_t s) {
  const int nthr = a.tile_w * a.tile_h / 2;
  a.vec_grads = ((reinterpret_cast<uintptr_t>(a.g_mean2d) & 7) == 0 &&
                 (reinterpret_cast<uintptr_t>(a.g_cov2d) & 15) == 0)
                    ? 1
                    : 0;
  a.batch = nthr < GSX_BWD2_BATCH ? nthr : GSX_BWD2_BATCH;
  const size_t smem = bwd2_smem<C>(a.batch, nthr);
  static size_t attr_done = 0, attr_done_p = 0;
  cudaError_t e = ensure_smem(raster_backward2_kernel<C, MAXT, BATCHED, RGB>, smem, attr_done);
  if (e != cudaSuccess) return cuda_status(e, "raster_backward2 smem attribute");
  unsigned launch_grid = 0;
  if constexpr (BATCHED) {
    if (a.work_counter) {  // persistent grid over the batch's tiles
      auto kp = raster_backward2_kernel<C, MAXT, BATCHED, RGB, true>;
      e = ensure_smem(kp, smem, attr_done_p);
      if (e == cudaSuccess) e = raster_grid(kp, nthr, smem, grid, a, s, launch_grid);
      if (e != cudaSuccess) return cuda_status(e, "raster grid");
      count_launches(1);
      kp<<<launch_grid, nthr, smem, s>>>(a);
      return cuda_status(cudaGetLastError(), "raster_backward2_kernel launch");
    }
  }
  a.work_counter = nullptr;
  e = raster_grid(raster_backward2_kernel<C, MAXT, BATCHED, RGB>, nthr, smem, grid, a, s, launch_grid);
  if (e != cudaSuccess) return cuda_status(e, "raster grid");
  count_launches(1);
  raster_backward2_kernel<C, MAXT, BATCHED, RGB><<<launch_grid, nthr, smem, s>>>(a);
  return cuda_status(cudaGetLastError(), "raster_backward2_kernel launch");
}


template <int C, bool BATCHED>
int launch_bwd_t(const RasterArgs &a, int64_t grid, cudaStream_t s) {
  if (use_two_pixels(a)) {
    const int nthr = a.tile_w * a.tile_h / 2;
    return nthr <= 128   ? launch_bwd2_tt<C, 128, BATCHED>(a, grid, s)
           : nthr <= 256 ? launch_bwd2_tt<C, 256, BATCHED>(a, grid, s)
                         : launch_bwd2_tt<C, 512, BATCHED>(a, grid, s);
  }
  return block_threads(a) <= 256 ? launch_bwd_tt<C, 256, BATCHED>(a, grid, s)
                                 : launch_bwd_tt<C, 1024, BATCHED>(a, grid, s);
}

template <bool BATCHED>
int dispatch_fwd(const RasterArgs &a, int C, int64_t grid, cudaStream_t s) {
  switch (C) {
    case 1: return launch_fwd_t<1, BATCHED>(a, grid, s);
    case 2: return launch_fwd_t<2, BATCHED>(a, grid, s);
    case 3: return launch_fwd_t<3, BATCHED>(a, grid, s);
    case 4: return launch_fwd_t<4, BATCHED>(a, grid, s);
  }
  set_error("SH order C must be 1..4 (got %d)", C);
  return GSX_ERR_INVALID_ARG;
}

template <bool BATCHED>
int dispatch_bwd(const RasterArgs &a, int C, int64_t grid, cudaStream_t s) {
  switch (C) {
    case 1: return launch_bwd_t<1, BATCHED>(a, grid, s);
    case 2: return launch_bwd_t<2, BATCHED>(a, grid, s);
    case 3: return launch_bwd_t<3, BATCHED>(a, grid, s);
    case 4: return launch_bwd_t<4, BATCHED>(a, grid, s);
  }
  set_error("SH order C must be 1..4 (got %d)", C);
  return GSX_ERR_INVALID_ARG;
}

}  // namespace

// Longest-processing-time-first order of the tiles for the raster passes:
// their grids run in ~13-18 waves of CTAs, and the tail is set by the heavy
// tiles (long lists) when they start late.  One CTA: a histogram of 256
// log-spaced length classes (8 per doubling), its exclusive scan from the
// longest class down, then each tile claims a slot in its class (lanes of a
// warp with the same class claim together).  Classes of the first
// kOrderCache tiles per thread stay in registers between the two passes.
constexpr int kOrderThreads = 1024, kOrderCache = 16;

__device__ __forceinline__ uint32_t length_class(const int32_t *__restrict__ start,
                                                 const int32_t *__restrict__ end, int tile) {
  const int32_t s0 = start[tile], e0 = end[tile];
  const uint32_t len = (s0 >= 0 && e0 > s0) ? (uint32_t)(e0 - s0) : 0u;
  // 8 classes per doubling of len + 1 (log2 with 3 mantissa bits); longest = class 0
  const uint32_t v = len + 1u;
  const int e = 31 - __clz(v);
  const uint32_t frac = e >= 3 ? (v >> (e - 3)) & 7u : (v << (3 - e)) & 7u;
  return 255u - ((uint32_t)e * 8u + frac);
}

__global__ void __launch_bounds__(kOrderThreads) tile_order_kernel(const int32_t *__restrict__ start,
                                                                   const int32_t *__restrict__ end,
                                                                   int32_t n_tiles,
                                                                   int32_t *__restrict__ order) {
  __shared__ uint32_t s_cnt[256];
  const int t = threadIdx.x, lane = t & 31;
  if (t < 256) s_cnt[t] = 0;
  __syncthreads();
  uint32_t cache[kOrderCache];
  const int rounds = (n_tiles + kOrderThreads - 1) / kOrderThreads;  // CTA-uniform
  // all cached rounds' loads first, so their latencies overlap
#pragma unroll
  for (int k = 0; k < kOrderCache; ++k) {
    const int i = k * kOrderThreads + t;
    cache[k] = i < n_tiles ? length_class(start, end, i) : 256u;
  }
  for (int k = 0; k < rounds; ++k) {
    const int i = k * kOrderThreads + t;
    uint32_t c = 256u;
    if (k < kOrderCache) {
#pragma unroll
      for (int q = 0; q < kOrderCache; ++q)
        if (q == k) c = cache[q];
    } else if (i < n_tiles) {
      c = length_class(start, end, i);
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, c);
    if (c < 256u && (peers & ((1u << lane) - 1u)) == 0) atomicAdd(&s_cnt[c], __popc(peers));
  }
  __syncthreads();
  if (t < 32) {  // exclusive scan of the 256 class counts, 8 per lane
    uint32_t v[8], sum = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      v[q] = s_cnt[8 * t + q];
      sum += v[q];
    }
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (t >= o) incl += y;
    }
    uint32_t run = incl - sum;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      s_cnt[8 * t + q] = run;
      run += v[q];
    }
  }
  __syncthreads();
  for (int k = 0; k < rounds; ++k) {
    const int i = k * kOrderThreads + t;
    uint32_t c = 256u;
    if (k < kOrderCache) {
#pragma unroll
      for (int q = 0; q < kOrderCache; ++q)
        if (q == k) c = cache[q];
    } else if (i < n_tiles) {
      c = length_class(start, end, i);
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, c);
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (c < 256u && lane == leader) base = atomicAdd(&s_cnt[c], __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (c < 256u) order[base + __popc(peers & ((1u << lane) - 1u))] = i;
  }
}

int launch_tile_order(const int32_t *start, const int32_t *end, int32_t n_tiles, int32_t *order,
                      cudaStream_t s) {
  if (n_tiles <= 0) return GSX_OK;
  count_launches(1);
  tile_order_kernel<<<1, kOrderThreads, 0, s>>>(start, end, n_tiles, order);
  return cuda_status(cudaGetLastError(), "tile_order_kernel launch");
}

int launch_raster_forward(const RasterArgs &a, int C, cudaStream_t s) {
  const int64_t grid = (int64_t)a.n_tiles_w * a.n_tiles_h;
  if (grid == 0) return GSX_OK;
  return dispatch_fwd<false>(a, C, grid, s);
}

int launch_raster_forward_rgb(const RasterArgs &a, cudaStream_t s) {
  const int64_t grid = (int64_t)a.n_tiles_w * a.n_tiles_h;
  if (grid == 0) return GSX_OK;
  if (use_two_pixels_fwd(a)) return launch_fwd2_t<1, false, true>(a, grid, s);
  return block_threads(a) <= 256 ? launch_fwd_tt<1, 256, false, false, true>(a, grid, s)
                                 : launch_fwd_tt<1, 1024, false, false, true>(a, grid, s);
}

int launch_raster_backward_rgb(const RasterArgs &a, cudaStream_t s) {
  const int64_t grid = (int64_t)a.n_tiles_w * a.n_tiles_h;
  if (grid == 0) return GSX_OK;
  if (use_two_pixels(a)) {
    const int nthr = a.tile_w * a.tile_h / 2;
    return nthr <= 128   ? launch_bwd2_tt<1, 128, false, true>(a, grid, s)
           : nthr <= 256 ? launch_bwd2_tt<1, 256, false, true>(a, grid, s)
                         : launch_bwd2_tt<1, 512, false, true>(a, grid, s);
  }
  return block_threads(a) <= 256 ? launch_bwd_tt<1, 256, false, true>(a, grid, s)
                                 : launch_bwd_tt<1, 1024, false, true>(a, grid, s);
}

int launch_raster_backward(const RasterArgs &a, int C, cudaStream_t s) {
  const int64_t grid = (int64_t)a.n_tiles_w * a.n_tiles_h;
  if (grid == 0) return GSX_OK;
  return dispatch_bwd<false>(a, C, grid, s);
}

int launch_raster_forward_batch(const RasterArgs &a, int C, int64_t total_tiles, cudaStream_t s) {
  if (total_tiles == 0) return GSX_OK;
  return dispatch_fwd<true>(a, C, total_tiles, s);
}

int launch_raster_backward_batch(const RasterArgs &a, int C, int64_t total_tiles, cudaStream_t s) {
  if (total_tiles == 0) return GSX_OK;
  return dispatch_bwd<true>(a, C, total_tiles, s);
}

__global__ void exp_selftest_kernel(const float *__restrict__ x, int64_t n, float *__restrict__ out,
                                    int variant) {
  const int64_t i = 2 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= n) return;
  const float a = x[i], b = i + 1 < n ? x[i + 1] : 0.0f;
  float ra, rb;
  if (variant == 0) {
    ra = gsx_expf(a);
    rb = gsx_expf(b);
  } else if (variant == 1) {
    ra = gsx_expf_nonpos(a);
    rb = gsx_expf_nonpos(b);
  } else {
    const float2 r = gsx_expf_nonpos2(make_float2(a, b));
    ra = r.x;
    rb = r.y;
  }
  out[i] = ra;
  if (i + 1 < n) out[i + 1] = rb;
}

int exp_selftest(const float *x, int64_t n, float *out, int variant, cudaStream_t s) {
  if (n <= 0) return GSX_OK;
  const int64_t pairs = (n + 1) / 2;
  count_launches(1);
  exp_selftest_kernel<<<(unsigned)((pairs + 255) / 256), 256, 0, s>>>(x, n, out, variant);
  return cuda_status(cudaGetLastError(), "exp_selftest_kernel launch");
}

int raster_wait_selftest(uint32_t limit, uint32_t *polls_dev, cudaStream_t s) {
  count_launches(1);
  bounded_wait_selftest_kernel<<<1, 32, 0, s>>>(limit, polls_dev);
  return cuda_status(cudaGetLastError(), "bounded_wait_selftest_kernel launch");
}

int raster_status(uint32_t *flags, int clear, cudaStream_t s) {
  cudaError_t e = cudaMemcpyFromSymbolAsync(flags, g_raster_flags, sizeof(uint32_t), 0,
                                            cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && clear && *flags) {
    const uint32_t zero = 0;
    e = cudaMemcpyToSymbolAsync(g_raster_flags, &zero, sizeof(uint32_t), 0,
                                cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  return cuda_status(e, "raster status");
}

}  // namespace gsx
