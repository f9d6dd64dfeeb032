// colors.cu -- opt-in per-Gaussian colours ("SH -> RGB in the projection").
//
// The reference evaluates the SH colour per pixel, from each pixel's ray
// (gs/src/include/vol_render_sh.h:139-141, 208-217); that stays the default.
// This file provides the common alternative in which each Gaussian gets one
// colour per view, from the direction camera centre -> mean:
//   dir = (mean - cam_pos) / |mean - cam_pos|,
//   rgb_ch = sigmoid(sum_k sh[ch, k] Y_k(dir))
// with the same SH basis polynomials and constants (shencoder.h:13-58) and
// the same sigmoid colour (shencoder.h:4-6).  The raster then composites the
// stored colours (raster.cu, RGB instantiations), and the backward below maps
// dL/drgb back to the SH coefficients and, through the direction, to the mean.
//
// One thread per Gaussian; culled Gaussians (counts[g] <= 0) get rgb = 0 and
// zero gradients.
#include "gsx_internal.cuh"

namespace gsx {

namespace {

// A value and its partial derivatives with respect to the three direction
// components, for differentiating the basis polynomials exactly.
struct D3 {
  float v, x, y, z;
};
__device__ __forceinline__ D3 d3c(float c) { return {c, 0.0f, 0.0f, 0.0f}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return {a.v + b.v, a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return {a.v - b.v, a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 operator*(float c, D3 a) { return {c * a.v, c * a.x, c * a.y, c * a.z}; }
__device__ __forceinline__ D3 operator*(D3 a, D3 b) {
  return {a.v * b.v, a.x * b.v + a.v * b.x, a.y * b.v + a.v * b.y, a.z * b.v + a.v * b.z};
}

template <typename T>
__device__ __forceinline__ T cst(float c);
template <>
__device__ __forceinline__ float cst<float>(float c) { return c; }
template <>
__device__ __forceinline__ D3 cst<D3>(float c) { return d3c(c); }

// Real SH basis of degree C - 1 at the unit direction (x, y, z), the
// polynomials of gs/src/include/shencoder.h:13-58.
template <int C, typename T>
__device__ __forceinline__ void sh_basis_dir(T x, T y, T z, T *Y) {
  Y[0] = cst<T>(0.28209479177387814f);
  if constexpr (C > 1) {
    Y[1] = -0.48860251190291987f * y;
    Y[2] = 0.48860251190291987f * z;
    Y[3] = -0.48860251190291987f * x;
  }
  if constexpr (C > 2) {
    const T xy = x * y, yz = y * z, xz = x * z, x2 = x * x, y2 = y * y, z2 = z * z;
    Y[4] = 1.0925484305920792f * xy;
    Y[5] = -1.0925484305920792f * yz;
    Y[6] = 0.94617469575755997f * z2 - cst<T>(0.31539156525251999f);
    Y[7] = -1.0925484305920792f * xz;
    Y[8] = 0.54627421529603959f * x2 - 0.54627421529603959f * y2;
    if constexpr (C > 3) {
      Y[9] = (0.59004358992664352f * y) * (y2 - 3.0f * x2);
      Y[10] = (2.8906114426405538f * xy) * z;
      Y[11] = (0.45704579946446572f * y) * (cst<T>(1.0f) - 5.0f * z2);
      Y[12] = (0.3731763325901154f * z) * (5.0f * z2 - cst<T>(3.0f));
      Y[13] = (0.45704579946446572f * x) * (cst<T>(1.0f) - 5.0f * z2);
      Y[14] = (1.4453057213202769f * z) * (x2 - y2);
      Y[15] = (0.59004358992664352f * x) * (3.0f * y2 - x2);
    }
  }
}

// Unit direction camera centre -> mean and its length (0 -> the zero vector).
__device__ __forceinline__ float view_dir(const float *m, float3 cam, float &dx, float &dy,
                                          float &dz) {
  const float ax = m[0] - cam.x, ay = m[1] - cam.y, az = m[2] - cam.z;
  const float len = sqrtf(fmaf(az, az, fmaf(ay, ay, ax * ax)));
  const float inv = len > 0.0f ? 1.0f / len : 0.0f;
  dx = ax * inv;
  dy = ay * inv;
  dz = az * inv;
  return len;
}

// One channel row of CC coefficients: 16-byte accesses when the row starts
// on a 16-byte boundary and CC is a multiple of 4 (C = 2, 4 with such a
// stride), else scalar ones.
template <int CC>
__device__ __forceinline__ void load_row(const float *__restrict__ p, bool vec, float (&v)[CC]) {
  if constexpr (CC % 4 == 0) {
    if (vec) {
#pragma unroll
      for (int k = 0; k < CC; k += 4) {
        const float4 q = *reinterpret_cast<const float4 *>(p + k);
        v[k] = q.x;
        v[k + 1] = q.y;
        v[k + 2] = q.z;
        v[k + 3] = q.w;
      }
      return;
    }
  }
#pragma unroll
  for (int k = 0; k < CC; ++k) v[k] = p[k];
}

template <int CC>
__device__ __forceinline__ void store_row(float *__restrict__ p, bool vec, const float (&v)[CC]) {
  if constexpr (CC % 4 == 0) {
    if (vec) {
#pragma unroll
      for (int k = 0; k < CC; k += 4)
        *reinterpret_cast<float4 *>(p + k) = make_float4(v[k], v[k + 1], v[k + 2], v[k + 3]);
      return;
    }
  }
#pragma unroll
  for (int k = 0; k < CC; ++k) p[k] = v[k];
}

template <int C>
__global__ void __launch_bounds__(256)
    colors_forward_kernel(int64_t n, const float *__restrict__ mean, const float *__restrict__ sh,
                          int sh_stride, float3 cam, const int32_t *__restrict__ counts,
                          float *__restrict__ rgb) {
  constexpr int CC = C * C;
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  float *o = rgb + 3 * g;
  if (counts && counts[g] <= 0) {
    o[0] = o[1] = o[2] = 0.0f;
    return;
  }
  float x, y, z;
  view_dir(mean + 3 * g, cam, x, y, z);
  float Y[CC];
  sh_basis_dir<C, float>(x, y, z, Y);
  const bool vec = ((sh_stride & 3) == 0) && ((reinterpret_cast<uintptr_t>(sh) & 15) == 0);
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    float v[CC];
    load_row<CC>(sh + (g * 3 + ch) * sh_stride, vec, v);
    float logit = 0.0f;
#pragma unroll
    for (int k = 0; k < CC; ++k) logit = fmaf(v[k], Y[k], logit);
    o[ch] = gsx_sigmoidf(logit);
  }
}

template <int C>
__global__ void __launch_bounds__(256)
    colors_backward_kernel(int64_t n, const float *__restrict__ mean, const float *__restrict__ sh,
                           int sh_stride, float3 cam, const int32_t *__restrict__ counts,
                           const float *__restrict__ rgb, const float *__restrict__ g_rgb,
                           float *__restrict__ g_sh, float *__restrict__ g_mean) {
  constexpr int CC = C * C;
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  if (counts && counts[g] <= 0) {
    for (int i = 0; i < 3 * sh_stride; ++i) g_sh[g * 3 * sh_stride + i] = 0.0f;
    return;
  }
  float x, y, z;
  const float len = view_dir(mean + 3 * g, cam, x, y, z);
  D3 Y[CC];
  sh_basis_dir<C, D3>(D3{x, 1.0f, 0.0f, 0.0f}, D3{y, 0.0f, 1.0f, 0.0f}, D3{z, 0.0f, 0.0f, 1.0f},
                      Y);
  float gx = 0.0f, gy = 0.0f, gz = 0.0f;  // dL/ddir
  const bool vec = ((sh_stride & 3) == 0) && ((reinterpret_cast<uintptr_t>(sh) & 15) == 0) &&
                   ((reinterpret_cast<uintptr_t>(g_sh) & 15) == 0);
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    const float c = rgb[3 * g + ch];
    const float dl = g_rgb[3 * g + ch] * (c * (1.0f - c));  // dL/dlogit
    float v[CC], gs[CC];
    load_row<CC>(sh + (g * 3 + ch) * sh_stride, vec, v);
#pragma unroll
    for (int k = 0; k < CC; ++k) {
      gs[k] = dl * Y[k].v;
      const float w = dl * v[k];
      gx = fmaf(w, Y[k].x, gx);
      gy = fmaf(w, Y[k].y, gy);
      gz = fmaf(w, Y[k].z, gz);
    }
    float *row = g_sh + (g * 3 + ch) * sh_stride;
    store_row<CC>(row, vec, gs);
    for (int k = CC; k < sh_stride; ++k) row[k] = 0.0f;
  }
  if (len > 0.0f) {  // d dir / d mean = (I - dir dir^T) / len
    const float dot = fmaf(z, gz, fmaf(y, gy, x * gx));
    float *gm = g_mean + 3 * g;
    gm[0] += (gx - x * dot) / len;
    gm[1] += (gy - y * dot) / len;
    gm[2] += (gz - z * dot) / len;
  }
}

float3 cam_pos(const float *p) { return make_float3(p[0], p[1], p[2]); }

}  // namespace

int launch_colors_forward(int64_t n, const float *mean, const float *sh, int sh_stride, int C,
                          const float *cam_pos_host, const int32_t *counts, float *rgb,
                          cudaStream_t s) {
  if (n == 0) return GSX_OK;
  const unsigned grid = (unsigned)((n + 255) / 256);
  const float3 cam = cam_pos(cam_pos_host);
  count_launches(1);
  switch (C) {
    case 1: colors_forward_kernel<1><<<grid, 256, 0, s>>>(n, mean, sh, sh_stride, cam, counts, rgb); break;
    case 2: colors_forward_kernel<2><<<grid, 256, 0, s>>>(n, mean, sh, sh_stride, cam, counts, rgb); break;
    case 3: colors_forward_kernel<3><<<grid, 256, 0, s>>>(n, mean, sh, sh_stride, cam, counts, rgb); break;
    case 4: colors_forward_kernel<4><<<grid, 256, 0, s>>>(n, mean, sh, sh_stride, cam, counts, rgb); break;
    default:
      set_error("SH order C must be 1..4 (got %d)", C);
      return GSX_ERR_INVALID_ARG;
  }
  return cuda_status(cudaGetLastError(), "colors_forward_kernel launch");
}

int launch_colors_backward(int64_t n, const float *mean, const float *sh, int sh_stride, int C,
                           const float *cam_pos_host, const int32_t *counts, const float *rgb,
                           const float *g_rgb, float *g_sh, float *g_mean, cudaStream_t s) {
  if (n == 0) return GSX_OK;
  const unsigned grid = (unsigned)((n + 255) / 256);
  const float3 cam = cam_pos(cam_pos_host);
  count_launches(1);
  switch (C) {
    case 1:
      colors_backward_kernel<1><<<grid, 256, 0, s>>>(n, mean, sh, sh_stride, cam, counts, rgb, g_rgb, g_sh, g_mean);
      break;
    case 2:
      colors_backward_kernel<2><<<grid, 256, 0, s>>>(n, mean, sh, sh_stride, cam, counts, rgb, g_rgb, g_sh, g_mean);
      break;
    case 3:
      colors_backward_kernel<3><<<grid, 256, 0, s>>>(n, mean, sh, sh_stride, cam, counts, rgb, g_rgb, g_sh, g_mean);
      break;
    case 4:
      colors_backward_kernel<4><<<grid, 256, 0, s>>>(n, mean, sh, sh_stride, cam, counts, rgb, g_rgb, g_sh, g_mean);
      break;
    default:
      set_error("SH order C must be 1..4 (got %d)", C);
      return GSX_ERR_INVALID_ARG;
  }
  return cuda_status(cudaGetLastError(), "colors_backward_kernel launch");
}

}  // namespace gsx
