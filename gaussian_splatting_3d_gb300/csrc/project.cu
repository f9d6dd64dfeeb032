// project.cu -- per-Gaussian passes: bounding-sphere culling (drop-in), the
// fused projection forward and its backward.
//
// Reference behaviour restated here:
//   culling      gs/src/include/culling.h:11-20, kernels.h:156-170
//   projection   gs/renderer.py:365-419 (project_pts, jacobian under no_grad,
//                cov2d = (J W Sigma W^T J^T)[:2,:2], mean2d = p_xy / p_z)
//   rotation     utils/transforms.py:31-45 (WXYZ quaternion normalised first,
//                M = R diag(s), Sigma = M M^T)
//   activations  utils/activations.py:13-19 (svec = exp, alpha = sigmoid)
//   AABB / count gs/culling.py:8-37, utils/camera.py:290-303
//
// One thread per Gaussian; every output row is written by the thread that
// owns it, so the pass is a single streaming read of 44 B and write of
// 48 B per Gaussian.
#include "ff_rot.cuh"
#include "gsx_internal.cuh"

namespace gsx {

namespace {

__global__ void cull_bsphere_kernel(int64_t n, const float *__restrict__ mean,
                                    const float *__restrict__ svec,
                                    const float *__restrict__ normal,
                                    const float *__restrict__ pts,
                                    uint8_t *__restrict__ mask, float thresh) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *s = svec + 3 * i;
  float r = fmaxf(fmaxf(s[0], s[1]), s[2]) * thresh;
  const float *m = mean + 3 * i;
  mask[i] = sphere_in_frustum(m[0], m[1], m[2], r, normal, pts) ? 1 : 0;
}

struct ProjCam {
  float W[3][3];  // W = R^T, W[i][j] = c2w[j][i]
  float t[3];
  float fx, fy, cx, cy;
  int32_t width, height;
  float normals[18], pts[18];
};

ProjCam make_proj_cam(const gsx_camera &c) {
  ProjCam p;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) p.W[i][j] = c.c2w[4 * j + i];
  p.t[0] = c.c2w[3];
  p.t[1] = c.c2w[7];
  p.t[2] = c.c2w[11];
  p.fx = c.fx;
  p.fy = c.fy;
  p.cx = c.cx;
  p.cy = c.cy;
  p.width = c.width;
  p.height = c.height;
  for (int k = 0; k < 18; ++k) {
    p.normals[k] = c.frustum_normals[k];
    p.pts[k] = c.frustum_pts[k];
  }
  return p;
}

struct Rot {
  float w, x, y, z;  // normalised quaternion
  float R[3][3];
};

__device__ __forceinline__ void quat_rot(const float4 q, Rot &o) {
  float n2 = fmaf(q.w, q.w, fmaf(q.z, q.z, fmaf(q.y, q.y, q.x * q.x)));
  float nrm = fmaxf(sqrtf(n2), 1e-12f);
  float w = q.x / nrm, x = q.y / nrm, y = q.z / nrm, z = q.w / nrm;
  o.w = w;
  o.x = x;
  o.y = y;
  o.z = z;
  float tx = 2.0f * x, ty = 2.0f * y, tz = 2.0f * z;
  float twx = tx * w, twy = ty * w, twz = tz * w;
  float txx = tx * x, txy = ty * x, txz = tz * x;
  float tyy = ty * y, tyz = tz * y, tzz = tz * z;
  o.R[0][0] = 1.0f - (tyy + tzz);
  o.R[0][1] = txy - twz;
  o.R[0][2] = txz + twy;
  o.R[1][0] = txy + twz;
  o.R[1][1] = 1.0f - (txx + tzz);
  o.R[1][2] = tyz - twx;
  o.R[2][0] = txz - twy;
  o.R[2][1] = tyz + twx;
  o.R[2][2] = 1.0f - (txx + tyy);
}

// One Gaussian through activation, cull, projection, covariance and AABB.
__device__ __forceinline__ void project_one(const ProjCam &cam, const float *__restrict__ mean,
                                            float4 q, const float *__restrict__ log_scale,
                                            const float *__restrict__ alpha_logit, int64_t g,
                                            float frustum_radius, float tile_radius, int32_t tile_w,
                                            int32_t tile_h, int32_t activated, float2 &o_mean2d,
                                            float4 &o_cov2d, float &o_depth, float &o_alpha,
                                            int4 &o_rect, int32_t &o_count) {
  const float m0 = mean[3 * g], m1 = mean[3 * g + 1], m2 = mean[3 * g + 2];
  float s0 = log_scale[3 * g], s1 = log_scale[3 * g + 1], s2 = log_scale[3 * g + 2];
  if (!activated) {
    s0 = gsx_expf(s0);
    s1 = gsx_expf(s1);
    s2 = gsx_expf(s2);
  }
  o_alpha = alpha_logit ? gsx_sigmoidf(alpha_logit[g]) : 0.0f;
  float r = fmaxf(fmaxf(s0, s1), s2) * frustum_radius;
  if (!sphere_in_frustum(m0, m1, m2, r, cam.normals, cam.pts)) {
    o_count = 0;
    o_rect = make_int4(0, 0, -1, -1);
    o_mean2d = make_float2(0.0f, 0.0f);
    o_cov2d = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    o_depth = 0.0f;
    return;
  }
  // p = W (x - t)
  float v0 = m0 - cam.t[0], v1 = m1 - cam.t[1], v2 = m2 - cam.t[2];
  float p[3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
    p[i] = fmaf(cam.W[i][2], v2, fmaf(cam.W[i][1], v1, cam.W[i][0] * v0));
  Rot rot;
  quat_rot(q, rot);
  const float sv[3] = {s0, s1, s2};
  float M[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) M[i][j] = sv[j] * rot.R[i][j];
  float S[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      S[i][k] = fmaf(M[i][2], M[k][2], fmaf(M[i][1], M[k][1], M[i][0] * M[k][0]));
  float iz = 1.0f / p[2];
  float j02 = (-p[0] / p[2]) / p[2];
  float j12 = (-p[1] / p[2]) / p[2];
  float A[2][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    A[0][k] = fmaf(j02, cam.W[2][k], iz * cam.W[0][k]);
    A[1][k] = fmaf(j12, cam.W[2][k], iz * cam.W[1][k]);
  }
  float T[2][3];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      T[i][k] = fmaf(A[i][2], S[2][k], fmaf(A[i][1], S[1][k], A[i][0] * S[0][k]));
  float cv[2][2];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int l = 0; l < 2; ++l)
      cv[i][l] = fmaf(T[i][2], A[l][2], fmaf(T[i][1], A[l][1], T[i][0] * A[l][0]));
  float mx = p[0] / p[2], my = p[1] / p[2];
  o_mean2d = make_float2(mx, my);
  o_cov2d = make_float4(cv[0][0], cv[0][1], cv[1][0], cv[1][1]);
  o_depth = p[2];
  float ax = sqrtf(tile_radius * cv[0][0]);
  float ay = sqrtf(tile_radius * cv[1][1]);
  float tlx = mx - ax, tly = my - ay, brx = mx + ax, bry = my + ay;
  float ptlx = tlx * cam.fx + cam.cx, ptly = tly * cam.fy + cam.cy;
  float pbrx = brx * cam.fx + cam.cx, pbry = bry * cam.fy + cam.cy;
  int32_t itlx = min(max(f2i_sat(ptlx), 0), cam.width - 1) / tile_w;
  int32_t itly = min(max(f2i_sat(ptly), 0), cam.height - 1) / tile_h;
  int32_t ibrx = min(max(f2i_sat(pbrx), 0), cam.width - 1) / tile_w;
  int32_t ibry = min(max(f2i_sat(pbry), 0), cam.height - 1) / tile_h;
  o_rect = make_int4(itlx, itly, ibrx, ibry);
  o_count = (ibrx - itlx + 1) * (ibry - itly + 1);
}

__global__ void __launch_bounds__(256)
    project_forward_kernel(int64_t n, const float *__restrict__ mean,
                           const float4 *__restrict__ qvec,
                           const float *__restrict__ log_scale,
                           const float *__restrict__ alpha_logit, const ProjCam cam,
                           float frustum_radius, float tile_radius, int32_t tile_w,
                           int32_t tile_h, int32_t activated,
                           float2 *__restrict__ mean2d, float4 *__restrict__ cov2d,
                           float *__restrict__ depth, float *__restrict__ alpha,
                           int4 *__restrict__ rect, int32_t *__restrict__ counts) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  project_one(cam, mean, qvec[g], log_scale, alpha_logit, g, frustum_radius, tile_radius, tile_w,
              tile_h, activated, mean2d[g], cov2d[g], depth[g], alpha[g], rect[g], counts[g]);
}

__device__ __forceinline__ ProjCam proj_cam_of(const gsx_camera &c) {
  ProjCam p;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) p.W[i][j] = c.c2w[4 * j + i];
  p.t[0] = c.c2w[3];
  p.t[1] = c.c2w[7];
  p.t[2] = c.c2w[11];
  p.fx = c.fx;
  p.fy = c.fy;
  p.cx = c.cx;
  p.cy = c.cy;
  p.width = c.width;
  p.height = c.height;
#pragma unroll
  for (int k = 0; k < 18; ++k) {
    p.normals[k] = c.frustum_normals[k];
    p.pts[k] = c.frustum_pts[k];
  }
  return p;
}

// All views of a batch: grid (Gaussian blocks, view); item = view's item
// offset + Gaussian index.
__global__ void __launch_bounds__(256)
    project_forward_batch_kernel(const gsx_batch_view *__restrict__ views, float frustum_radius,
                                 float tile_radius, float2 *__restrict__ mean2d,
                                 float4 *__restrict__ cov2d, float *__restrict__ depth,
                                 float *__restrict__ alpha, int4 *__restrict__ rect,
                                 int32_t *__restrict__ counts) {
  const gsx_batch_view &v = views[blockIdx.y];
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= v.n_gaussians) return;
  const int64_t item = v.item_offset + g;
  const ProjCam cam = proj_cam_of(v.cam);
  const float4 q = reinterpret_cast<const float4 *>(v.qvec)[g];
  project_one(cam, v.mean, q, v.log_scale, v.alpha_logit, g, frustum_radius, tile_radius, v.tile_w,
              v.tile_h, 0, mean2d[item], cov2d[item], depth[item], alpha[item], rect[item],
              counts[item]);
}

// Parity-mode backward of the projection (depth detached, J constant):
// the part that depends on the view.  Adds dL/dmean (through
// mean2d = p_xy / p_z) into gm and dL/dSigma = A^T Gc A into GS.
// Rotation, scales and M = R diag(s) of one Gaussian (as project_one makes
// them), shared by the view-dependent and the parameter parts of the backward.
struct Frame {
  Rot rot;
  float s[3];
  float M[3][3];
};

__device__ __forceinline__ void make_frame(float4 q, const float *__restrict__ log_scale,
                                           int64_t g, Frame &f) {
  quat_rot(q, f.rot);  // the normalised quaternion (and R for a degenerate q)
  f.s[0] = gsx_expf(log_scale[3 * g]);
  f.s[1] = gsx_expf(log_scale[3 * g + 1]);
  f.s[2] = gsx_expf(log_scale[3 * g + 2]);
  if (!frame_ff(q, f.s, f.rot.R, f.M)) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) f.M[i][j] = f.s[j] * f.rot.R[i][j];
  }
}

__device__ __forceinline__ void world_cov(const Frame &f, float (&S)[3][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      S[i][k] = fmaf(f.M[i][2], f.M[k][2], fmaf(f.M[i][1], f.M[k][1], f.M[i][0] * f.M[k][0]));
}

// The view-dependent part of the backward for one (Gaussian, view):
// dL/dmean2d and dL/dcov2d -> dL/dmean (added into gm) and dL/dSigma (added
// into GS).  flags = 0 is the reference's gradient: mean2d = p_xy / stopgrad(z)
// and J constant (gs/renderer.py:365-377, 408-417).  GSX_GRAD_DEPTH adds the
// z term of mean2d, GSX_GRAD_JACOBIAN the dependence of J on p (Sig = the
// world covariance, needed only then).
__device__ __forceinline__ void accum_view_grad(const ProjCam &cam, float m0, float m1, float m2,
                                                float2 gm2, float4 gc, int32_t flags,
                                                const float (&Sig)[3][3], float (&gm)[3],
                                                float (&GS)[3][3]) {
  float v0 = m0 - cam.t[0], v1 = m1 - cam.t[1], v2 = m2 - cam.t[2];
  float p[3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
    p[i] = fmaf(cam.W[i][2], v2, fmaf(cam.W[i][1], v1, cam.W[i][0] * v0));
  float gp0 = gm2.x / p[2], gp1 = gm2.y / p[2], gp2 = 0.0f;
  float iz = 1.0f / p[2];
  float j02 = (-p[0] / p[2]) / p[2];
  float j12 = (-p[1] / p[2]) / p[2];
  float A[2][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    A[0][k] = fmaf(j02, cam.W[2][k], iz * cam.W[0][k]);
    A[1][k] = fmaf(j12, cam.W[2][k], iz * cam.W[1][k]);
  }
  float B[2][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    B[0][k] = fmaf(gc.y, A[1][k], gc.x * A[0][k]);
    B[1][k] = fmaf(gc.w, A[1][k], gc.z * A[0][k]);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) GS[i][k] += fmaf(A[1][i], B[1][k], A[0][i] * B[0][k]);
  if (flags & (GSX_GRAD_DEPTH | GSX_GRAD_JACOBIAN)) {
    const float iz2 = iz * iz;
    if (flags & GSX_GRAD_DEPTH) gp2 = -fmaf(gm2.x, p[0], gm2.y * p[1]) * iz2;
    if (flags & GSX_GRAD_JACOBIAN) {
      // cov2d = A Sig A^T, A = J(p) W: dL/dA = (Gc + Gc^T) A Sig, dL/dJ = dL/dA W^T,
      // with J00 = J11 = 1/z, J02 = -x/z^2, J12 = -y/z^2
      float AS[2][3];
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int k = 0; k < 3; ++k)
          AS[a][k] = fmaf(A[a][2], Sig[2][k], fmaf(A[a][1], Sig[1][k], A[a][0] * Sig[0][k]));
      const float h00 = 2.0f * gc.x, h01 = gc.y + gc.z, h11 = 2.0f * gc.w;
      float gA[2][3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        gA[0][k] = fmaf(h01, AS[1][k], h00 * AS[0][k]);
        gA[1][k] = fmaf(h11, AS[1][k], h01 * AS[0][k]);
      }
      float gJ[2][3];
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          gJ[a][j] = fmaf(gA[a][2], cam.W[j][2], fmaf(gA[a][1], cam.W[j][1], gA[a][0] * cam.W[j][0]));
      gp0 = fmaf(-gJ[0][2], iz2, gp0);
      gp1 = fmaf(-gJ[1][2], iz2, gp1);
      const float t2 = 2.0f * fmaf(gJ[0][2], p[0], gJ[1][2] * p[1]) * (iz2 * iz);
      gp2 = fmaf(-(gJ[0][0] + gJ[1][1]), iz2, gp2 + t2);
    }
#pragma unroll
    for (int j = 0; j < 3; ++j)
      gm[j] += fmaf(cam.W[2][j], gp2, fmaf(cam.W[1][j], gp1, cam.W[0][j] * gp0));
  } else {
#pragma unroll
    for (int j = 0; j < 3; ++j) gm[j] += fmaf(cam.W[1][j], gp1, cam.W[0][j] * gp0);
  }
}

// The view-independent part: dL/dSigma -> quaternion and log-scale, and the
// opacity logit (zero where min(alpha, 0.99) clamps, with GSX_GRAD_CLAMP).
__device__ __forceinline__ void finish_param_grad(const Frame &f, float4 q, float alpha_logit,
                                                  int64_t g, const float (&GS)[3][3],
                                                  float g_alpha, int32_t flags,
                                                  float *__restrict__ g_logs, float4 &g_q,
                                                  float &g_al) {
  const Rot &rot = f.rot;
  float GR[3][3];
  float gsc[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      float acc = 0.0f;
#pragma unroll
      for (int k = 0; k < 3; ++k) acc = fmaf(GS[i][k] + GS[k][i], f.M[k][j], acc);
      GR[i][j] = acc * f.s[j];
      gsc[j] = fmaf(acc, rot.R[i][j], gsc[j]);
    }
#pragma unroll
  for (int j = 0; j < 3; ++j) g_logs[3 * g + j] = gsc[j] * f.s[j];
  const float w = rot.w, x = rot.x, y = rot.y, z = rot.z;
  float gw = 2.0f * (-z * GR[0][1] + y * GR[0][2] + z * GR[1][0] - x * GR[1][2] -
                     y * GR[2][0] + x * GR[2][1]);
  float gx = 2.0f * (y * GR[0][1] + z * GR[0][2] + y * GR[1][0] - 2.0f * x * GR[1][1] -
                     w * GR[1][2] + z * GR[2][0] + w * GR[2][1] - 2.0f * x * GR[2][2]);
  float gy = 2.0f * (-2.0f * y * GR[0][0] + x * GR[0][1] + w * GR[0][2] + x * GR[1][0] +
                     z * GR[1][2] - w * GR[2][0] + z * GR[2][1] - 2.0f * y * GR[2][2]);
  float gz = 2.0f * (-2.0f * z * GR[0][0] - w * GR[0][1] + x * GR[0][2] + w * GR[1][0] -
                     2.0f * z * GR[1][1] + y * GR[1][2] + x * GR[2][0] + y * GR[2][1]);
  float nq = sqrtf(fmaf(q.w, q.w, fmaf(q.z, q.z, fmaf(q.y, q.y, q.x * q.x))));
  if (nq > 1e-12f) {
    float dp = gw * w + gx * x + gy * y + gz * z;
    g_q = make_float4((gw - dp * w) / nq, (gx - dp * x) / nq, (gy - dp * y) / nq,
                      (gz - dp * z) / nq);
  } else {
    g_q = make_float4(gw / 1e-12f, gx / 1e-12f, gy / 1e-12f, gz / 1e-12f);
  }
  float a = gsx_sigmoidf(alpha_logit);
  g_al = ((flags & GSX_GRAD_CLAMP) && a > 0.99f) ? 0.0f : g_alpha * (a * (1.0f - a));
}

__global__ void __launch_bounds__(256)
    project_backward_kernel(int64_t n, const float *__restrict__ mean,
                            const float4 *__restrict__ qvec,
                            const float *__restrict__ log_scale,
                            const float *__restrict__ alpha_logit, const ProjCam cam,
                            const int32_t *__restrict__ counts,
                            const float2 *__restrict__ g_mean2d,
                            const float4 *__restrict__ g_cov2d,
                            const float *__restrict__ g_alpha,
                            float *__restrict__ g_mean, float4 *__restrict__ g_qvec,
                            float *__restrict__ g_logs,
                            float *__restrict__ g_alpha_logit, int32_t flags) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  if (counts[g] == 0) {
    g_mean[3 * g] = 0.0f;
    g_mean[3 * g + 1] = 0.0f;
    g_mean[3 * g + 2] = 0.0f;
    g_logs[3 * g] = 0.0f;
    g_logs[3 * g + 1] = 0.0f;
    g_logs[3 * g + 2] = 0.0f;
    g_qvec[g] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    g_alpha_logit[g] = 0.0f;
    return;
  }
  const float4 q = qvec[g];
  Frame f;
  make_frame(q, log_scale, g, f);
  float Sig[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
  if (flags & GSX_GRAD_JACOBIAN) world_cov(f, Sig);
  float gm[3] = {0.0f, 0.0f, 0.0f};
  float GS[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
  accum_view_grad(cam, mean[3 * g], mean[3 * g + 1], mean[3 * g + 2], g_mean2d[g], g_cov2d[g],
                  flags, Sig, gm, GS);
#pragma unroll
  for (int j = 0; j < 3; ++j) g_mean[3 * g + j] = gm[j];
  finish_param_grad(f, q, alpha_logit[g], g, GS, g_alpha[g], flags, g_logs, g_qvec[g],
                    g_alpha_logit[g]);
}

// Batched backward for views that share one scene (views[0]'s): per
// Gaussian, sum the view-dependent parts over every view that saw it, then
// back-propagate once through the rotation, scales and opacity.
__global__ void __launch_bounds__(256)
    project_backward_batch_kernel(const gsx_batch_view *__restrict__ views, int32_t n_views,
                                  const int32_t *__restrict__ counts,
                                  const float2 *__restrict__ g_mean2d,
                                  const float4 *__restrict__ g_cov2d,
                                  const float *__restrict__ g_alpha, int32_t flags) {
  const gsx_batch_view &v0 = views[0];
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= v0.n_gaussians) return;
  const float m0 = v0.mean[3 * g], m1 = v0.mean[3 * g + 1], m2 = v0.mean[3 * g + 2];
  float gm[3] = {0.0f, 0.0f, 0.0f};
  float GS[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
  float ga = 0.0f;
  const float4 q = reinterpret_cast<const float4 *>(v0.qvec)[g];
  float Sig[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
  if (flags & GSX_GRAD_JACOBIAN) {  // the frame is made again after the view loop: fewer live registers in it
    Frame f0;
    make_frame(q, v0.log_scale, g, f0);
    world_cov(f0, Sig);
  }
  bool seen = false;
  for (int vi = 0; vi < n_views; ++vi) {
    const int64_t item = views[vi].item_offset + g;
    if (counts[item] == 0) continue;
    seen = true;
    accum_view_grad(proj_cam_of(views[vi].cam), m0, m1, m2, g_mean2d[item], g_cov2d[item], flags,
                    Sig, gm, GS);
    ga += g_alpha[item];
  }
  float4 *g_qvec = reinterpret_cast<float4 *>(v0.g_qvec);
  if (!seen) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      v0.g_mean[3 * g + j] = 0.0f;
      v0.g_log_scale[3 * g + j] = 0.0f;
    }
    g_qvec[g] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    v0.g_alpha_logit[g] = 0.0f;
    return;
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) v0.g_mean[3 * g + j] = gm[j];
  float4 gq;
  float gal;
  Frame f;
  make_frame(q, v0.log_scale, g, f);
  finish_param_grad(f, q, v0.alpha_logit[g], g, GS, ga, flags, v0.g_log_scale, gq, gal);
  g_qvec[g] = gq;
  v0.g_alpha_logit[g] = gal;
}

inline unsigned grid_for(int64_t n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

}  // namespace

int launch_project_forward_batch(const gsx_batch_view *views, int32_t n_views, int64_t max_n,
                                 float frustum_radius, float tile_radius, float *mean2d,
                                 float *cov2d, float *depth, float *alpha, int32_t *rect,
                                 int32_t *counts, cudaStream_t s) {
  if (max_n == 0 || n_views == 0) return GSX_OK;
  count_launches(1);
  project_forward_batch_kernel<<<dim3(grid_for(max_n, 256), (unsigned)n_views), 256, 0, s>>>(
      views, frustum_radius, tile_radius, reinterpret_cast<float2 *>(mean2d),
      reinterpret_cast<float4 *>(cov2d), depth, alpha, reinterpret_cast<int4 *>(rect), counts);
  return cuda_status(cudaGetLastError(), "project_forward_batch_kernel launch");
}

int launch_project_backward_batch(const gsx_batch_view *views, int32_t n_views, int64_t n,
                                  const int32_t *counts, const float *g_mean2d,
                                  const float *g_cov2d, const float *g_alpha, int32_t flags,
                                  cudaStream_t s) {
  if (n == 0 || n_views == 0) return GSX_OK;
  count_launches(1);
  project_backward_batch_kernel<<<grid_for(n, 256), 256, 0, s>>>(
      views, n_views, counts, reinterpret_cast<const float2 *>(g_mean2d),
      reinterpret_cast<const float4 *>(g_cov2d), g_alpha, flags);
  return cuda_status(cudaGetLastError(), "project_backward_batch_kernel launch");
}

int launch_cull_bsphere(int64_t n, const float *mean, const float *svec,
                        const float *normal, const float *pts, uint8_t *mask,
                        float thresh, cudaStream_t s) {
  if (n == 0) return GSX_OK;
  count_launches(1);
  cull_bsphere_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, mean, svec, normal, pts,
                                                        mask, thresh);
  return cuda_status(cudaGetLastError(), "cull_bsphere_kernel launch");
}

int launch_project_forward(int64_t n, const float *mean, const float *qvec,
                           const float *log_scale, const float *alpha_logit,
                           const gsx_camera &cam, float frustum_radius,
                           float tile_radius, int32_t tile_w, int32_t tile_h,
                           int32_t scales_are_activated, float *mean2d,
                           float *cov2d, float *depth, float *alpha, int32_t *rect,
                           int32_t *counts, cudaStream_t s) {
  if (n == 0) return GSX_OK;
  count_launches(1);
  project_forward_kernel<<<grid_for(n, 256), 256, 0, s>>>(
      n, mean, reinterpret_cast<const float4 *>(qvec), log_scale, alpha_logit,
      make_proj_cam(cam), frustum_radius, tile_radius, tile_w, tile_h,
      scales_are_activated, reinterpret_cast<float2 *>(mean2d),
      reinterpret_cast<float4 *>(cov2d), depth, alpha, reinterpret_cast<int4 *>(rect),
      counts);
  return cuda_status(cudaGetLastError(), "project_forward_kernel launch");
}

int launch_project_backward(int64_t n, const float *mean, const float *qvec,
                            const float *log_scale, const float *alpha_logit,
                            const gsx_camera &cam, const int32_t *counts,
                            const float *g_mean2d, const float *g_cov2d,
                            const float *g_alpha, float *g_mean, float *g_qvec,
                            float *g_logs, float *g_alpha_logit, int32_t flags,
                            cudaStream_t s) {
  if (n == 0) return GSX_OK;
  count_launches(1);
  project_backward_kernel<<<grid_for(n, 256), 256, 0, s>>>(
      n, mean, reinterpret_cast<const float4 *>(qvec), log_scale, alpha_logit,
      make_proj_cam(cam), counts, reinterpret_cast<const float2 *>(g_mean2d),
      reinterpret_cast<const float4 *>(g_cov2d), g_alpha, g_mean,
      reinterpret_cast<float4 *>(g_qvec), g_logs, g_alpha_logit, flags);
  return cuda_status(cudaGetLastError(), "project_backward_kernel launch");
}

}  // namespace gsx
