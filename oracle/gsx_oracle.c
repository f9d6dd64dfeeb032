/*
 * gsx_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A plain-C CPU restatement of the reference's SH Gaussian-splatting path
 * (heheyas/gaussian_splatting_3d).  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load this library, and only as the checker or
 * as the timed CPU baseline; the product never links or calls it.
 *
 * Parity pin: the npz files under tests/golden hold outputs of the reference itself run on
 * a CPU (its Python projection imported as-is, its CUDA kernels compiled from
 * their own sources under a CPU emulation of the CUDA runtime; recipe in
 * oracle/build_ref.py and tests/golden/make_golden.py).  tests/test_oracle_golden.py
 * checks every function below against those vectors.
 *
 * Arithmetic contract.  The CUDA kernels of the product follow exactly the
 * same operation sequence, so for the same inputs the oracle and the kernels
 * agree bit for bit on every threshold decision (cull, 1/255 skip, T_thresh
 * stop, AABB truncation) and on the forward image:
 *   - fmaf() is written wherever nvcc would contract the reference's a*b+c;
 *     the file is compiled with -ffp-contract=off so nothing else fuses;
 *   - division and sqrtf are IEEE correctly rounded on both sides;
 *   - exp is gsx_expf() below (Cody-Waite range reduction with a two-part
 *     ln2 -- the float split SLEEF publishes --, degree-7 Taylor polynomial
 *     in Horner form, 2^j scaling through the
 *     exponent bits; flush to +0 below -87).  The reference calls CUDA's
 *     expf; gsx_expf stays within 2 ulp of the correctly rounded value on the
 *     range the path uses (checked against libm in the tests).
 *   - the 2D-Gaussian gradient is evaluated in double, as the reference does
 *     (gs/src/include/kernels.h:394-418).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MIN_RENDER_ALPHA (1.0f / 255.0f) /* gs/src/include/common.h:89 */

/* ------------------------------------------------------------------------ */
/* exp and sigmoid                                                           */
/* ------------------------------------------------------------------------ */

static inline float f_from_bits(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint32_t bits_from_f(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

float orc_expf(float x) {
  if (!(x > -87.0f)) return (x != x) ? x : 0.0f;
  if (x > 88.75f) return INFINITY;
  /* j = round-to-nearest-even(x * log2(e)) via the 1.5*2^23 shifter */
  float t = fmaf(x, 1.44269502162933349609375f, 12582912.0f);
  float j = t - 12582912.0f;
  float r = fmaf(j, -0.693145751953125f, x);          /* ln2 high part, exact product */
  r = fmaf(j, -1.428606765330187045e-06f, r);           /* ln2 low part */
  float p = 1.98412698412698412e-04f;                  /* 1/7! */
  p = fmaf(p, r, 1.38888888888888889e-03f);             /* 1/6! */
  p = fmaf(p, r, 8.33333333333333333e-03f);             /* 1/5! */
  p = fmaf(p, r, 4.16666666666666667e-02f);             /* 1/4! */
  p = fmaf(p, r, 1.66666666666666667e-01f);             /* 1/3! */
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  int ji = (int)j;
  if (ji > 127) { p = p * 2.0f; ji -= 1; }
  return p * f_from_bits((uint32_t)(ji + 127) << 23);
}

/* gs/src/include/shencoder.h:4 */
static inline float sigmoidf_(float x) { return 1.0f / (1.0f + orc_expf(-x)); }

/* ------------------------------------------------------------------------ */
/* frustum culling: gs/src/include/culling.h:11-20, kernels.h:156-170        */
/* ------------------------------------------------------------------------ */

static inline float dot3_pts(const float *q, const float *p, const float *n) {
  float dx = q[0] - p[0], dy = q[1] - p[1], dz = q[2] - p[2];
  return fmaf(dz, n[2], fmaf(dy, n[1], dx * n[0]));
}

static inline int sphere_in_frustum(const float *m, float r, const float *normals,
                                    const float *pts) {
  for (int i = 0; i < 6; ++i)
    if (!(dot3_pts(m, pts + 3 * i, normals + 3 * i) > -r)) return 0;
  return 1;
}

/* mask[i] = sphere(mean_i, max(svec_i) * thresh) intersects all 6 half-spaces */
void orc_cull_bsphere(int64_t n, const float *mean, const float *svec,
                      const float *normals, const float *pts, float thresh,
                      uint8_t *mask) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const float *s = svec + 3 * i;
    float r = fmaxf(fmaxf(s[0], s[1]), s[2]) * thresh;
    mask[i] = (uint8_t)sphere_in_frustum(mean + 3 * i, r, normals, pts);
  }
}

/* ------------------------------------------------------------------------ */
/* projection (gs/renderer.py:365-419, utils/transforms.py:31-45 with the    */
/* WXYZ quaternion normalised first, gs/culling.py:8-37,                     */
/* utils/camera.py:290-303) fused with culling, as one per-Gaussian pass.    */
/* ------------------------------------------------------------------------ */

/* float -> int32 the way the GPU converts: truncate, saturate, NaN -> 0 */
static inline int32_t f2i_sat(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return INT32_MAX;
  if (f < -2147483648.0f) return INT32_MIN;
  return (int32_t)f;
}

static inline int32_t clampi(int32_t v, int32_t lo, int32_t hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}

typedef struct {
  float c2w[12];
  float fx, fy, cx, cy;
  int32_t width, height;
  float normals[18];
  float pts[18];
} orc_camera;

/*
 * For every Gaussian: activation (svec = exp(log_s), alpha = sigmoid(logit)),
 * bounding-sphere cull, projection to normalised image coordinates,
 * 2D covariance (J and W constant), the AABB tile rectangle and its key
 * count.  Culled Gaussians get count 0 and rect (0,0,-1,-1).
 * If log_scale_is_svec != 0, `log_s` already holds activated scales.
 */
void orc_project(int64_t n, const float *mean, const float *qvec,
                 const float *log_s, const float *alpha_logit,
                 const orc_camera *cam, float frustum_radius, float tile_radius,
                 int32_t tile_w, int32_t tile_h, int32_t log_scale_is_svec,
                 uint8_t *mask, float *mean2d, float *cov2d, float *depth,
                 float *alpha, int32_t *rect, int32_t *counts) {
  const float *c = cam->c2w;
  /* W = R^T, W[i][j] = c2w[j][i] */
  float Wm[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Wm[i][j] = c[4 * j + i];
  const float t0 = c[3], t1 = c[7], t2 = c[11];
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < n; ++g) {
    const float *m = mean + 3 * g;
    const float *ls = log_s + 3 * g;
    float s0, s1, s2;
    if (log_scale_is_svec) { s0 = ls[0]; s1 = ls[1]; s2 = ls[2]; }
    else { s0 = orc_expf(ls[0]); s1 = orc_expf(ls[1]); s2 = orc_expf(ls[2]); }
    if (alpha) alpha[g] = alpha_logit ? sigmoidf_(alpha_logit[g]) : 0.0f;
    float r = fmaxf(fmaxf(s0, s1), s2) * frustum_radius;
    int vis = sphere_in_frustum(m, r, cam->normals, cam->pts);
    if (mask) mask[g] = (uint8_t)vis;
    int32_t *rc = rect + 4 * g;
    if (!vis) {
      counts[g] = 0;
      rc[0] = 0; rc[1] = 0; rc[2] = -1; rc[3] = -1;
      mean2d[2 * g] = 0.0f; mean2d[2 * g + 1] = 0.0f;
      for (int k = 0; k < 4; ++k) cov2d[4 * g + k] = 0.0f;
      depth[g] = 0.0f;
      continue;
    }
    /* p = W (x - t)   (gs/renderer.py:380-387) */
    float v0 = m[0] - t0, v1 = m[1] - t1, v2 = m[2] - t2;
    float p[3];
    for (int i = 0; i < 3; ++i)
      p[i] = fmaf(Wm[i][2], v2, fmaf(Wm[i][1], v1, Wm[i][0] * v0));
    /* R(q) with q normalised (WXYZ) */
    const float *q = qvec + 4 * g;
    float n2 = fmaf(q[3], q[3], fmaf(q[2], q[2], fmaf(q[1], q[1], q[0] * q[0])));
    float nrm = fmaxf(sqrtf(n2), 1e-12f);
    float w = q[0] / nrm, x = q[1] / nrm, y = q[2] / nrm, z = q[3] / nrm;
    float tx = 2.0f * x, ty = 2.0f * y, tz = 2.0f * z;
    float twx = tx * w, twy = ty * w, twz = tz * w;
    float txx = tx * x, txy = ty * x, txz = tz * x;
    float tyy = ty * y, tyz = tz * y, tzz = tz * z;
    float R[3][3] = {{1.0f - (tyy + tzz), txy - twz, txz + twy},
                     {txy + twz, 1.0f - (txx + tzz), tyz - twx},
                     {txz - twy, tyz + twx, 1.0f - (txx + tyy)}};
    /* M = R diag(s)  (svec.unsqueeze(-2) * R) ; Sigma = M M^T */
    float sv[3] = {s0, s1, s2};
    float M[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) M[i][j] = sv[j] * R[i][j];
    float S[3][3];
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k)
        S[i][k] = fmaf(M[i][2], M[k][2], fmaf(M[i][1], M[k][1], M[i][0] * M[k][0]));
    /* J rows 0,1 (gs/renderer.py:365-377); JW = J W */
    float iz = 1.0f / p[2];
    float j02 = (-p[0] / p[2]) / p[2];
    float j12 = (-p[1] / p[2]) / p[2];
    float A[2][3];
    for (int k = 0; k < 3; ++k) {
      A[0][k] = fmaf(j02, Wm[2][k], iz * Wm[0][k]);
      A[1][k] = fmaf(j12, Wm[2][k], iz * Wm[1][k]);
    }
    /* cov2d = (A S A^T)[:2,:2] via T = A S */
    float T[2][3];
    for (int i = 0; i < 2; ++i)
      for (int k = 0; k < 3; ++k)
        T[i][k] = fmaf(A[i][2], S[2][k], fmaf(A[i][1], S[1][k], A[i][0] * S[0][k]));
    float cv[2][2];
    for (int i = 0; i < 2; ++i)
      for (int l = 0; l < 2; ++l)
        cv[i][l] = fmaf(T[i][2], A[l][2], fmaf(T[i][1], A[l][1], T[i][0] * A[l][0]));
    float mx = p[0] / p[2], my = p[1] / p[2];
    mean2d[2 * g] = mx; mean2d[2 * g + 1] = my;
    cov2d[4 * g + 0] = cv[0][0]; cov2d[4 * g + 1] = cv[0][1];
    cov2d[4 * g + 2] = cv[1][0]; cov2d[4 * g + 3] = cv[1][1];
    depth[g] = p[2];
    /* AABB (gs/culling.py:17-31): separate multiply and add, int32 truncation,
       clamp to the image, floor-divide by the tile size */
    float ax = sqrtf(tile_radius * cv[0][0]);
    float ay = sqrtf(tile_radius * cv[1][1]);
    float tlx = mx - ax, tly = my - ay, brx = mx + ax, bry = my + ay;
    float ptlx = tlx * cam->fx + cam->cx;
    float ptly = tly * cam->fy + cam->cy;
    float pbrx = brx * cam->fx + cam->cx;
    float pbry = bry * cam->fy + cam->cy;
    int32_t itlx = clampi(f2i_sat(ptlx), 0, cam->width - 1) / tile_w;
    int32_t itly = clampi(f2i_sat(ptly), 0, cam->height - 1) / tile_h;
    int32_t ibrx = clampi(f2i_sat(pbrx), 0, cam->width - 1) / tile_w;
    int32_t ibry = clampi(f2i_sat(pbry), 0, cam->height - 1) / tile_h;
    rc[0] = itlx; rc[1] = itly; rc[2] = ibrx; rc[3] = ibry;
    counts[g] = (ibrx - itlx + 1) * (ibry - itly + 1);
  }
}

/* ------------------------------------------------------------------------ */
/* tile binning: gs/src/include/aabb_culling.h:15-41 (key emission),         */
/* :235-241 (stable 64-bit sort), :70-103 (start / end)                       */
/* ------------------------------------------------------------------------ */

typedef struct { uint64_t key; int32_t id; } orc_kv;

static int kv_cmp(const void *a, const void *b) {
  const orc_kv *x = (const orc_kv *)a, *y = (const orc_kv *)b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  return (x->id > y->id) - (x->id < y->id); /* canonical order of equal keys */
}

/*
 * Keys (tile_id << 32) | bits(depth) for every Gaussian and every tile of its
 * rectangle (rect = tlx, tly, brx, bry in tile units), sorted ascending as
 * unsigned 64-bit values; equal keys ordered by Gaussian index.  Writes up to
 * `cap` ids and the sorted keys (if keys_out != NULL); start/end get the first
 * and one-past-last position of each tile, -1 for empty tiles.  rect_stride is
 * 4 for (tl, br) packed rows, or 2 when tl and br are separate [M,2] arrays
 * passed as rect and rect_br.  Returns K; nothing but start/end is written
 * when K > cap.
 */
int64_t orc_bin(int64_t n, const int32_t *rect_tl, const int32_t *rect_br,
                int32_t rect_stride, const float *depth, int32_t n_tiles_h,
                int32_t n_tiles_w, int64_t cap, int32_t *ids_out,
                uint64_t *keys_out, int32_t *start, int32_t *end) {
  int64_t T = (int64_t)n_tiles_h * n_tiles_w;
  int64_t K = 0;
  for (int64_t g = 0; g < n; ++g) {
    const int32_t *tl = rect_tl + rect_stride * g;
    const int32_t *br = rect_br + rect_stride * g;
    int64_t w = (int64_t)br[0] - tl[0] + 1, h = (int64_t)br[1] - tl[1] + 1;
    if (w > 0 && h > 0) K += w * h;
  }
  for (int64_t t = 0; t < T; ++t) { start[t] = -1; end[t] = -1; }
  if (K > cap) return K;
  orc_kv *kv = (orc_kv *)malloc(sizeof(orc_kv) * (size_t)(K > 0 ? K : 1));
  int64_t pos = 0;
  for (int64_t g = 0; g < n; ++g) {
    const int32_t *tl = rect_tl + rect_stride * g;
    const int32_t *br = rect_br + rect_stride * g;
    uint32_t db = bits_from_f(depth[g]);
    for (int32_t i = tl[0]; i <= br[0]; ++i)      /* x outer */
      for (int32_t j = tl[1]; j <= br[1]; ++j) {  /* y inner */
        uint32_t tile = (uint32_t)(j * n_tiles_w + i);
        kv[pos].key = ((uint64_t)tile << 32) | db;
        kv[pos].id = (int32_t)g;
        ++pos;
      }
  }
  qsort(kv, (size_t)K, sizeof(orc_kv), kv_cmp);
  for (int64_t k = 0; k < K; ++k) {
    ids_out[k] = kv[k].id;
    if (keys_out) keys_out[k] = kv[k].key;
    int32_t t = (int32_t)(kv[k].key >> 32);
    if (k == 0 || (int32_t)(kv[k - 1].key >> 32) != t) start[t] = (int32_t)k;
    if (k == K - 1 || (int32_t)(kv[k + 1].key >> 32) != t) end[t] = (int32_t)(k + 1);
  }
  free(kv);
  return K;
}

/* ------------------------------------------------------------------------ */
/* SH raster: gs/src/include/vol_render_sh.h:48-65 (direction with the        */
/* reference's c2w row stride of 3), shencoder.h:13-58 (basis),               */
/* vol_render_sh.h:98-248 (forward), :268-455 (backward)                      */
/* ------------------------------------------------------------------------ */

typedef struct {
  int32_t width, height, tile_w, tile_h, n_tiles_w, n_tiles_h;
  int32_t C, sh_stride; /* SH order (degree + 1) and floats per channel */
  float T_thresh;
} orc_raster_params;

static inline void pixel_pos(const float *topleft, float psx, float psy, int gx,
                             int gy, float *px, float *py) {
  *px = fmaf((float)gx, psx, topleft[0]);
  *py = fmaf((float)gy, psy, topleft[1]);
}

static void sh_basis(const float *c2w, float px, float py, int C, float *Y) {
  /* direction = c2w read as float3 rows of the flat 12-float array */
  float d[3];
  for (int r = 0; r < 3; ++r) {
    const float *row = c2w + 3 * r;
    d[r] = fmaf(row[2], 1.0f, fmaf(row[1], py, row[0] * px));
  }
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

/* the 2D Gaussian: gs/src/include/kernels.h:172-193 */
static inline float gauss2d(const float *m, const float *cv, float px, float py) {
  float c0 = cv[0], c1 = cv[1], c2 = cv[2], c3 = cv[3];
  float det = fmaf(c0, c3, -(c1 * c2));
  float x = px - m[0], y = py - m[1];
  float tmpx = fmaf(x, c3, -(y * c2));
  float tmpy = fmaf(-x, c1, y * c0);
  float radial = fmaf(tmpx, x, tmpy * y);
  radial = radial / det;
  if (radial < 0.0f) radial = 1000.0f;
  return orc_expf(-0.5f * radial);
}

static inline float sh_dot(const float *sh, const float *Y, int CC) {
  float s = 0.0f;
  for (int k = 0; k < CC; ++k) s = fmaf(sh[k], Y[k], s);
  return s;
}

/* The forward with an optional background (out += T_final * bg), alpha map
 * (1 - T_final) and depth map (sum of T a G z): no reference counterpart
 * (its background variant, vol_render_bg.h, does not compile). */
void orc_render_fwd_ex(const orc_raster_params *P, const float *mean, const float *cov,
                       const float *sh, const float *alpha, const int32_t *start,
                       const int32_t *end, const int32_t *ids, const float *topleft,
                       const float *c2w, float psx, float psy, float *out, const float *bg,
                       const float *depth, float *alpha_out, float *depth_out) {
  const int C = P->C, CC = C * C, S = P->sh_stride;
  const int64_t T = (int64_t)P->n_tiles_w * P->n_tiles_h;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t t = 0; t < T; ++t) {
    const int empty = start[t] == -1 || end[t] - start[t] == 0;
    if (empty && !bg && !alpha_out && !depth_out) continue;
    int n = empty ? 0 : end[t] - start[t];
    int bx = (int)(t % P->n_tiles_w), by = (int)(t / P->n_tiles_w);
    for (int ly = 0; ly < P->tile_h; ++ly)
      for (int lx = 0; lx < P->tile_w; ++lx) {
        int gx = bx * P->tile_w + lx, gy = by * P->tile_h + ly;
        if (gx >= P->width || gy >= P->height) continue;
        float px, py, Y[16];
        pixel_pos(topleft, psx, psy, gx, gy, &px, &py);
        sh_basis(c2w, px, py, C, Y);
        float o[3] = {0.0f, 0.0f, 0.0f}, Tr = 1.0f, dsum = 0.0f;
        for (int i = 0; i < n; ++i) {
          if (Tr < P->T_thresh) break;
          int g = ids[start[t] + i];
          float a = fminf(alpha[g], 0.99f);
          float coeff = a * Tr;
          float G = gauss2d(mean + 2 * g, cov + 4 * g, px, py);
          coeff = coeff * G;
          if (a * G < MIN_RENDER_ALPHA) continue;
          if (isnan(coeff)) coeff = 0.0f;
          for (int ch = 0; ch < 3; ++ch) {
            float y = sigmoidf_(sh_dot(sh + ((int64_t)3 * g + ch) * S, Y, CC));
            if (isnan(y * coeff)) y = 0.0f;
            o[ch] = fmaf(coeff, y, o[ch]);
          }
          if (depth_out) dsum = fmaf(coeff, depth[g], dsum);
          Tr = Tr * fmaf(-a, G, 1.0f);
        }
        const int64_t pix = (int64_t)gy * P->width + gx;
        if (bg)
          for (int ch = 0; ch < 3; ++ch) o[ch] = fmaf(Tr, bg[ch], o[ch]);
        float *dst = out + 3 * pix;
        dst[0] = o[0]; dst[1] = o[1]; dst[2] = o[2];
        if (alpha_out) alpha_out[pix] = 1.0f - Tr;
        if (depth_out) depth_out[pix] = dsum;
      }
  }
}

void orc_render_fwd(const orc_raster_params *P, const float *mean, const float *cov,
                    const float *sh, const float *alpha, const int32_t *start,
                    const int32_t *end, const int32_t *ids, const float *topleft,
                    const float *c2w, float psx, float psy, float *out) {
  orc_render_fwd_ex(P, mean, cov, sh, alpha, start, end, ids, topleft, c2w, psx, psy, out, NULL,
                    NULL, NULL, NULL);
}

static inline void atomic_addf(float *p, float v) {
#pragma omp atomic
  *p += v;
}

/*
 * Backward (reference order: front-to-back recompute; per contributing pair
 * dL/dsh, dL/d(aG) through (final - out)/(1 - aG), the 2D-Gaussian gradient in
 * double, dL/dalpha).  Gradients are added into grad_* (caller zeroes them).
 * grad_cov receives the same value in slots 1 and 2, as the reference does.
 */
void orc_render_bwd(const orc_raster_params *P, const float *mean, const float *cov,
                    const float *sh, const float *alpha, const int32_t *start,
                    const int32_t *end, const int32_t *ids, const float *topleft,
                    const float *c2w, float psx, float psy, const float *out,
                    const float *grad_out, float *grad_mean, float *grad_cov,
                    float *grad_sh, float *grad_alpha) {
  const int C = P->C, CC = C * C, S = P->sh_stride;
  const int64_t T = (int64_t)P->n_tiles_w * P->n_tiles_h;
  const int NV = 7 + 3 * CC; /* per-Gaussian: mean 2, cov 4, alpha 1, sh 3CC */
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t t = 0; t < T; ++t) {
    if (start[t] == -1) continue;
    int n = end[t] - start[t];
    if (n == 0) continue;
    double *acc = (double *)calloc((size_t)n * NV, sizeof(double));
    int bx = (int)(t % P->n_tiles_w), by = (int)(t / P->n_tiles_w);
    for (int ly = 0; ly < P->tile_h; ++ly)
      for (int lx = 0; lx < P->tile_w; ++lx) {
        int gx = bx * P->tile_w + lx, gy = by * P->tile_h + ly;
        if (gx >= P->width || gy >= P->height) continue;
        float px, py, Y[16];
        pixel_pos(topleft, psx, psy, gx, gy, &px, &py);
        sh_basis(c2w, px, py, C, Y);
        int64_t pix = 3 * ((int64_t)gy * P->width + gx);
        float fin[3] = {out[pix], out[pix + 1], out[pix + 2]};
        float go[3] = {grad_out[pix], grad_out[pix + 1], grad_out[pix + 2]};
        float o[3] = {0.0f, 0.0f, 0.0f}, Tr = 1.0f;
        for (int i = 0; i < n; ++i) {
          if (Tr < P->T_thresh) break;
          int g = ids[start[t] + i];
          const float *m = mean + 2 * g, *cv = cov + 4 * g;
          float a = fminf(alpha[g], 0.99f);
          float G = gauss2d(m, cv, px, py);
          if (a * G < MIN_RENDER_ALPHA) continue;
          float coeff = a * Tr * G;
          if (isnan(coeff)) coeff = 0.0f;
          float y[3];
          for (int ch = 0; ch < 3; ++ch) {
            y[ch] = sigmoidf_(sh_dot(sh + ((int64_t)3 * g + ch) * S, Y, CC));
            if (isnan(y[ch] * coeff)) y[ch] = 0.0f;
            o[ch] = fmaf(coeff, y[ch], o[ch]);
          }
          double *A = acc + (size_t)i * NV;
          for (int ch = 0; ch < 3; ++ch) {
            float wgt = coeff * (y[ch] * (1.0f - y[ch])) * go[ch];
            for (int k = 0; k < CC; ++k) A[7 + ch * CC + k] += (double)(wgt * Y[k]);
          }
          float one_m = fmaf(-a, G, 1.0f);
          float Pg = 0.0f;
          for (int ch = 0; ch < 3; ++ch) {
            float qv = (fin[ch] - o[ch]) / one_m;
            Pg = fmaf(go[ch], fmaf(y[ch], Tr, -qv), Pg);
          }
          /* kernels.h:394-418 in double */
          double dg = (double)(Pg * a * G);
          double c0 = cv[0], c1 = cv[1], c2 = cv[2], c3 = cv[3];
          double det = c0 * c3 - c1 * c2;
          double x = (double)(px - m[0]), yy = (double)(py - m[1]);
          double tmpx = (x * c3 - yy * c2) / det;
          double tmpy = (-x * c1 + yy * c0) / det;
          A[0] += (float)(dg * tmpx);
          A[1] += (float)(dg * tmpy);
          A[2] += 0.5 * (float)(dg * tmpx * tmpx);
          A[3] += 0.5 * (float)(dg * tmpx * tmpy);
          A[4] += 0.5 * (float)(dg * tmpy * tmpx);
          A[5] += 0.5 * (float)(dg * tmpy * tmpy);
          A[6] += (double)(Pg * G);
          Tr = Tr * one_m;
        }
      }
    for (int i = 0; i < n; ++i) {
      int g = ids[start[t] + i];
      const double *A = acc + (size_t)i * NV;
      atomic_addf(grad_mean + 2 * g, (float)A[0]);
      atomic_addf(grad_mean + 2 * g + 1, (float)A[1]);
      for (int k = 0; k < 4; ++k) atomic_addf(grad_cov + 4 * g + k, (float)A[2 + k]);
      atomic_addf(grad_alpha + g, (float)A[6]);
      for (int ch = 0; ch < 3; ++ch)
        for (int k = 0; k < CC; ++k)
          atomic_addf(grad_sh + ((int64_t)3 * g + ch) * S + k, (float)A[7 + ch * CC + k]);
    }
    free(acc);
  }
}

/* ------------------------------------------------------------------------ */
/* projection backward: the autograd of gs/renderer.py:390-419 through      */
/* kornia's normalised-quaternion rotation, svec = exp(.) and                 */
/* alpha = sigmoid(.) (utils/activations.py).  Evaluated in double.           */
/* flags = 0 is the reference's gradient: depth detached                      */
/* (mean2d = p_xy / stopgrad(p_z), gs/renderer.py:408-417), J constant        */
/* (@torch.no_grad jacobian, gs/renderer.py:365-377) and the opacity clamp    */
/* min(alpha, 0.99) ignored (vol_render_sh.h:346).  ORC_GRAD_DEPTH adds the   */
/* z term of mean2d (the reference's depth_detach=False), ORC_GRAD_JACOBIAN   */
/* the dependence of J on the camera-space mean, ORC_GRAD_CLAMP a zero        */
/* opacity gradient where the clamp is active: all three give the true        */
/* derivative of the rendered image.                                          */
/* ------------------------------------------------------------------------ */
#define ORC_GRAD_DEPTH 1
#define ORC_GRAD_JACOBIAN 2
#define ORC_GRAD_CLAMP 4
void orc_project_bwd(int64_t n, const float *mean, const float *qvec,
                     const float *log_s, const float *alpha_logit,
                     const orc_camera *cam, const uint8_t *mask,
                     const float *g_mean2d, const float *g_cov2d,
                     const float *g_alpha, float *g_mean, float *g_qvec,
                     float *g_logs, float *g_alpha_logit, int32_t flags) {
  const float *c = cam->c2w;
  double Wm[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Wm[i][j] = c[4 * j + i];
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < n; ++g) {
    for (int k = 0; k < 3; ++k) { g_mean[3 * g + k] = 0.0f; g_logs[3 * g + k] = 0.0f; }
    for (int k = 0; k < 4; ++k) g_qvec[4 * g + k] = 0.0f;
    g_alpha_logit[g] = 0.0f;
    if (!mask[g]) continue;
    const float *m = mean + 3 * g;
    double v[3] = {(double)m[0] - c[3], (double)m[1] - c[7], (double)m[2] - c[11]};
    double p[3];
    for (int i = 0; i < 3; ++i) p[i] = Wm[i][0] * v[0] + Wm[i][1] * v[1] + Wm[i][2] * v[2];
    /* mean2d = p_xy / z: dL/dp_xy = g / z (z detached unless ORC_GRAD_DEPTH) */
    const double gm2[2] = {g_mean2d[2 * g], g_mean2d[2 * g + 1]};
    double gp[3] = {gm2[0] / p[2], gm2[1] / p[2], 0.0};
    if (flags & ORC_GRAD_DEPTH) gp[2] = -(gm2[0] * p[0] + gm2[1] * p[1]) / (p[2] * p[2]);
    /* A = first two rows of J W */
    double iz = 1.0 / p[2], j02 = -p[0] / p[2] / p[2], j12 = -p[1] / p[2] / p[2];
    double A[2][3];
    for (int k = 0; k < 3; ++k) {
      A[0][k] = iz * Wm[0][k] + j02 * Wm[2][k];
      A[1][k] = iz * Wm[1][k] + j12 * Wm[2][k];
    }
    /* dL/dSigma = A^T Gc A */
    const float *gc = g_cov2d + 4 * g;
    double Gc[2][2] = {{gc[0], gc[1]}, {gc[2], gc[3]}};
    double GS[3][3];
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k) {
        double acc = 0.0;
        for (int a = 0; a < 2; ++a)
          for (int b = 0; b < 2; ++b) acc += A[a][i] * Gc[a][b] * A[b][k];
        GS[i][k] = acc;
      }
    const float *q = qvec + 4 * g;
    double qn2 = (double)q[0] * q[0] + (double)q[1] * q[1] + (double)q[2] * q[2] + (double)q[3] * q[3];
    double nq = sqrt(qn2);
    double nrm = nq > 1e-12 ? nq : 1e-12;
    double w = q[0] / nrm, x = q[1] / nrm, y = q[2] / nrm, z = q[3] / nrm;
    double R[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)},
                      {2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)},
                      {2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)}};
    const float *ls = log_s + 3 * g;
    double s[3] = {exp((double)ls[0]), exp((double)ls[1]), exp((double)ls[2])};
    double M[3][3], GM[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) M[i][j] = R[i][j] * s[j];
    if (flags & ORC_GRAD_JACOBIAN) {
      /* cov2d = A Sigma A^T with A = J(p) W: dL/dA = (Gc + Gc^T) A Sigma,
         dL/dJ = dL/dA W^T; J00 = J11 = 1/z, J02 = -x/z^2, J12 = -y/z^2 */
      double Sig[3][3], AS[2][3], gA[2][3], gJ[2][3];
      for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k)
          Sig[i][k] = M[i][0] * M[k][0] + M[i][1] * M[k][1] + M[i][2] * M[k][2];
      for (int a = 0; a < 2; ++a)
        for (int k = 0; k < 3; ++k)
          AS[a][k] = A[a][0] * Sig[0][k] + A[a][1] * Sig[1][k] + A[a][2] * Sig[2][k];
      for (int a = 0; a < 2; ++a)
        for (int k = 0; k < 3; ++k)
          gA[a][k] = (Gc[a][0] + Gc[0][a]) * AS[0][k] + (Gc[a][1] + Gc[1][a]) * AS[1][k];
      for (int a = 0; a < 2; ++a)
        for (int j = 0; j < 3; ++j)
          gJ[a][j] = gA[a][0] * Wm[j][0] + gA[a][1] * Wm[j][1] + gA[a][2] * Wm[j][2];
      const double iz2 = iz * iz;
      gp[0] += -gJ[0][2] * iz2;
      gp[1] += -gJ[1][2] * iz2;
      gp[2] += -(gJ[0][0] + gJ[1][1]) * iz2 + 2.0 * (gJ[0][2] * p[0] + gJ[1][2] * p[1]) * iz2 * iz;
    }
    for (int j = 0; j < 3; ++j)
      g_mean[3 * g + j] = (float)(Wm[0][j] * gp[0] + Wm[1][j] * gp[1] + Wm[2][j] * gp[2]);
    /* Sigma = M M^T, M = R diag(s): dL/dM = (GS + GS^T) M */
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double acc = 0.0;
        for (int k = 0; k < 3; ++k) acc += (GS[i][k] + GS[k][i]) * M[k][j];
        GM[i][j] = acc;
      }
    /* M_ij = R_ij s_j */
    double GR[3][3], gs[3] = {0, 0, 0};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        GR[i][j] = GM[i][j] * s[j];
        gs[j] += GM[i][j] * R[i][j];
      }
    for (int j = 0; j < 3; ++j) g_logs[3 * g + j] = (float)(gs[j] * s[j]);
    /* dR/d(w,x,y,z) for the unit quaternion */
    double gw = 2 * (-z * GR[0][1] + y * GR[0][2] + z * GR[1][0] - x * GR[1][2] - y * GR[2][0] + x * GR[2][1]);
    double gx = 2 * (y * GR[0][1] + z * GR[0][2] + y * GR[1][0] - 2 * x * GR[1][1] - w * GR[1][2] + z * GR[2][0] + w * GR[2][1] - 2 * x * GR[2][2]);
    double gy = 2 * (-2 * y * GR[0][0] + x * GR[0][1] + w * GR[0][2] + x * GR[1][0] + z * GR[1][2] - w * GR[2][0] + z * GR[2][1] - 2 * y * GR[2][2]);
    double gz = 2 * (-2 * z * GR[0][0] - w * GR[0][1] + x * GR[0][2] + w * GR[1][0] - 2 * z * GR[1][1] + y * GR[1][2] + x * GR[2][0] + y * GR[2][1]);
    /* through q / max(|q|, eps) */
    double gu[4] = {gw, gx, gy, gz}, u[4] = {w, x, y, z};
    if (nq > 1e-12) {
      double dotp = gu[0] * u[0] + gu[1] * u[1] + gu[2] * u[2] + gu[3] * u[3];
      for (int k = 0; k < 4; ++k) g_qvec[4 * g + k] = (float)((gu[k] - dotp * u[k]) / nq);
    } else {
      for (int k = 0; k < 4; ++k) g_qvec[4 * g + k] = (float)(gu[k] / 1e-12);
    }
    double sa = 1.0 / (1.0 + exp(-(double)alpha_logit[g]));
    /* the renderer uses min(alpha, 0.99) with alpha the float sigmoid */
    const int clamped = (flags & ORC_GRAD_CLAMP) && sigmoidf_(alpha_logit[g]) > 0.99f;
    g_alpha_logit[g] = clamped ? 0.0f : (float)(g_alpha[g] * sa * (1.0 - sa));
  }
}

int32_t orc_num_threads(void) {
#ifdef _OPENMP
  return (int32_t)omp_get_max_threads();
#else
  return 1;
#endif
}
