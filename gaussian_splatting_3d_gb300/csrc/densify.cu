// densify.cu -- per-Gaussian statistics for adaptive density control and the
// split / clone rewrite of the parameter arrays.
//
// Reference behaviour restated (gs/sh_renderer.py):
//   visit counts        :216        cnt[mask] += 1 for the Gaussians that
//                                   survive frustum culling
//   gradient statistic  :602-623    grad_mean = max(grad_mean, |g|) or
//                                   grad_mean += |g|, g = mean.grad (all
//                                   Gaussians) or mean_2d.grad (visible ones)
//   split / clone       :426-540    select by the statistic (optionally divided
//                                   by cnt + 1e-5) and max(scale) > thresh;
//                                   new arrays = [Gaussians not split, in
//                                   order] ++ [clones, in order] ++ [split
//                                   samples, copy 0 of every split Gaussian
//                                   then copy 1]; a split sample is
//                                   mean + R(q)^T (n * scale), n ~ N(0, 1),
//                                   with log-scale - log(shrink)
//
// The normal draws come from a counter-based generator (a 64-bit mix of
// (seed, Gaussian, copy, axis) -> two uniforms -> Box-Muller), so a split is
// reproducible for a seed; the reference draws them with torch.randn.
#include "gsx_internal.cuh"

namespace gsx {

namespace {

__global__ void count_visible_kernel(int64_t n, const int32_t *__restrict__ counts,
                                     int32_t *__restrict__ cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && counts[i] > 0) cnt[i] += 1;
}

__global__ void accumulate_norm_kernel(int64_t n, const float *__restrict__ grad, int dim,
                                       const int32_t *__restrict__ counts,
                                       float *__restrict__ accum, int reduce_max) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (counts && counts[i] <= 0) return;
  float s = 0.0f;
  for (int d = 0; d < dim; ++d) s = fmaf(grad[dim * i + d], grad[dim * i + d], s);
  const float v = sqrtf(s);
  accum[i] = reduce_max ? fmaxf(accum[i], v) : accum[i] + v;
}

// Class of each Gaussian: 0 keep, 1 clone, 2 split.
__global__ void classify_kernel(int64_t n, const float *__restrict__ accum,
                                const int32_t *__restrict__ cnt,
                                const float *__restrict__ log_scale, float grad_thresh,
                                float scale_thresh, int divide_by_count,
                                uint8_t *__restrict__ cls) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float stat = accum[i];
  if (divide_by_count) stat = stat / ((float)cnt[i] + 1e-5f);
  uint8_t c = 0;
  if (stat > grad_thresh) {
    bool large = false;
    for (int d = 0; d < 3; ++d) large = large || (gsx_expf(log_scale[3 * i + d]) > scale_thresh);
    c = large ? 2 : 1;
  }
  cls[i] = c;
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// One standard normal for (seed, gaussian, copy, axis): Box-Muller on two
// 24-bit uniforms in (0, 1].
__device__ __forceinline__ float normal_draw(uint64_t seed, int64_t g, int copy, int axis) {
  const uint64_t h = mix64(seed ^ mix64(((uint64_t)g << 3) | ((uint64_t)copy << 2) | (uint64_t)axis));
  const float u1 = ((float)(h >> 40) + 1.0f) * (1.0f / 16777216.0f);
  const float u2 = (float)((h >> 16) & 0xffffffull) * (1.0f / 16777216.0f);
  return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}

// Writes the rewritten arrays.  pos_keep/pos_clone/pos_split are exclusive
// prefix counts of the classes (keep includes clone sources: every Gaussian
// that is not split stays).
__global__ void rewrite_kernel(int64_t n, const uint8_t *__restrict__ cls,
                               const int64_t *__restrict__ pos_stay,
                               const int64_t *__restrict__ pos_clone,
                               const int64_t *__restrict__ pos_split, int64_t n_stay,
                               int64_t n_clone, int64_t n_split, const float *__restrict__ mean,
                               const float *__restrict__ qvec, const float *__restrict__ log_scale,
                               const float *__restrict__ sh, int sh_len,
                               const float *__restrict__ alpha_logit, float log_shrink,
                               uint64_t seed, float *__restrict__ o_mean,
                               float *__restrict__ o_qvec, float *__restrict__ o_log_scale,
                               float *__restrict__ o_sh, float *__restrict__ o_alpha) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint8_t c = cls[i];
  auto copy_to = [&](int64_t d, const float *m, const float *ls) {
    for (int k = 0; k < 3; ++k) o_mean[3 * d + k] = m[k];
    for (int k = 0; k < 4; ++k) o_qvec[4 * d + k] = qvec[4 * i + k];
    for (int k = 0; k < 3; ++k) o_log_scale[3 * d + k] = ls[k];
    for (int k = 0; k < sh_len; ++k) o_sh[(int64_t)sh_len * d + k] = sh[(int64_t)sh_len * i + k];
    o_alpha[d] = alpha_logit[i];
  };
  const float *m = mean + 3 * i, *ls = log_scale + 3 * i;
  if (c != 2) copy_to(pos_stay[i], m, ls);
  if (c == 1) copy_to(n_stay + pos_clone[i], m, ls);
  if (c == 2) {
    // R(q) of the normalised WXYZ quaternion; the sample uses its transpose
    const float qw = qvec[4 * i], qx = qvec[4 * i + 1], qy = qvec[4 * i + 2], qz = qvec[4 * i + 3];
    const float nq = fmaxf(sqrtf(qw * qw + qx * qx + qy * qy + qz * qz), 1e-12f);
    const float w = qw / nq, x = qx / nq, y = qy / nq, z = qz / nq;
    const float R[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)},
                           {2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)},
                           {2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)}};
    float s[3], nls[3];
    for (int k = 0; k < 3; ++k) {
      s[k] = gsx_expf(ls[k]);
      nls[k] = logf(s[k]) - log_shrink;
    }
    for (int copy = 0; copy < 2; ++copy) {
      float v[3], nm[3];
      for (int k = 0; k < 3; ++k) v[k] = normal_draw(seed, i, copy, k) * s[k];
      for (int r = 0; r < 3; ++r) nm[r] = m[r] + (R[0][r] * v[0] + R[1][r] * v[1] + R[2][r] * v[2]);
      copy_to(n_stay + n_clone + copy * n_split + pos_split[i], nm, nls);
    }
  }
}

inline unsigned blocks(int64_t n) { return (unsigned)((n + 255) / 256); }

}  // namespace

int launch_count_visible(int64_t n, const int32_t *counts, int32_t *cnt, cudaStream_t s) {
  if (n == 0) return GSX_OK;
  count_launches(1);
  count_visible_kernel<<<blocks(n), 256, 0, s>>>(n, counts, cnt);
  return cuda_status(cudaGetLastError(), "count_visible_kernel launch");
}

int launch_accumulate_norm(int64_t n, const float *grad, int dim, const int32_t *counts,
                           float *accum, int reduce_max, cudaStream_t s) {
  if (n == 0) return GSX_OK;
  count_launches(1);
  accumulate_norm_kernel<<<blocks(n), 256, 0, s>>>(n, grad, dim, counts, accum, reduce_max);
  return cuda_status(cudaGetLastError(), "accumulate_norm_kernel launch");
}

int launch_classify(int64_t n, const float *accum, const int32_t *cnt, const float *log_scale,
                    float grad_thresh, float scale_thresh, int divide_by_count, uint8_t *cls,
                    cudaStream_t s) {
  if (n == 0) return GSX_OK;
  count_launches(1);
  classify_kernel<<<blocks(n), 256, 0, s>>>(n, accum, cnt, log_scale, grad_thresh, scale_thresh,
                                            divide_by_count, cls);
  return cuda_status(cudaGetLastError(), "classify_kernel launch");
}

int launch_rewrite(int64_t n, const uint8_t *cls, const int64_t *pos_stay, const int64_t *pos_clone,
                   const int64_t *pos_split, int64_t n_stay, int64_t n_clone, int64_t n_split,
                   const float *mean, const float *qvec, const float *log_scale, const float *sh,
                   int sh_len, const float *alpha_logit, float log_shrink, uint64_t seed,
                   float *o_mean, float *o_qvec, float *o_log_scale, float *o_sh, float *o_alpha,
                   cudaStream_t s) {
  if (n == 0) return GSX_OK;
  count_launches(1);
  rewrite_kernel<<<blocks(n), 256, 0, s>>>(n, cls, pos_stay, pos_clone, pos_split, n_stay, n_clone,
                                           n_split, mean, qvec, log_scale, sh, sh_len, alpha_logit,
                                           log_shrink, seed, o_mean, o_qvec, o_log_scale, o_sh,
                                           o_alpha);
  return cuda_status(cudaGetLastError(), "rewrite_kernel launch");
}

}  // namespace gsx
