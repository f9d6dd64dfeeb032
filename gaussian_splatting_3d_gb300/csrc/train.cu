// train.cu -- the training step around the renderer: the photometric loss
// and its image gradient, and the Adam update of the parameter arrays.
//
// Loss (utils/loss.py:5-24): L = m * SSIM_loss(out, gt) + (1 - m) * base(out,
// gt), base = L1 or L2 (mean), SSIM_loss = mean(clamp((1 - SSIM) / 2, 0, 1))
// over channels and pixels, with kornia's published SSIM: an 11x11 (any odd
// size) normalised Gaussian window of sigma 1.5 applied per channel with
// reflected borders ("same" size), C1 = 0.01^2, C2 = 0.03^2,
// SSIM = (2 mu1 mu2 + C1)(2 s12 + C2) / ((mu1^2 + mu2^2 + C1)(s1 + s2 + C2) + eps).
// The gradient with respect to `out` runs the window filter's adjoint
// (reflection folded back onto the border pixels), so it is the exact
// derivative of that loss.  Images are HWC float32 [H, W, 3].
//
// Adam (gs/sh_renderer.py:720-729 builds torch.optim.Adam with per-group
// learning rates, betas (0.9, 0.99)): per element, in torch's order,
//   m += (1 - b1) (g - m);  v = b2 v + (1 - b2) g^2
//   p -= (lr / (1 - b1^t)) * m / (sqrt(v) / sqrt(1 - b2^t) + eps)
// over all parameter groups in one launch.
#include "gsx_internal.cuh"

namespace gsx {

namespace {

constexpr int kMaxWin = 31;

struct Window {
  float k[kMaxWin];
  int r;  // radius: window = 2r + 1
};

__device__ __forceinline__ int reflect(int m, int n) {
  if (m < 0) return -m;
  if (m > n - 1) return 2 * (n - 1) - m;
  return m;
}

// Row (horizontal) pass over the five maps x, y, x^2, y^2, x*y of one channel
// plane; out: [5][H][W] per channel.
__global__ void ssim_rows_kernel(const float *__restrict__ x, const float *__restrict__ y, int H,
                                 int W, const Window win, float *__restrict__ out) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t P = (int64_t)H * W;
  if (idx >= 3 * P) return;
  const int ch = (int)(idx / P);
  const int64_t p = idx - (int64_t)ch * P;
  const int row = (int)(p / W), col = (int)(p - (int64_t)row * W);
  float a[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  for (int d = -win.r; d <= win.r; ++d) {
    const int c = reflect(col + d, W);
    const int64_t q = 3 * ((int64_t)row * W + c) + ch;
    const float xv = x[q], yv = y[q], kk = win.k[d + win.r];
    a[0] = fmaf(kk, xv, a[0]);
    a[1] = fmaf(kk, yv, a[1]);
    a[2] = fmaf(kk, xv * xv, a[2]);
    a[3] = fmaf(kk, yv * yv, a[3]);
    a[4] = fmaf(kk, xv * yv, a[4]);
  }
  for (int m = 0; m < 5; ++m) out[((int64_t)ch * 5 + m) * P + p] = a[m];
}

// Column pass, then SSIM and the partial derivatives of the per-element loss
// with respect to the filtered maps mu1 (A), E[x^2] (B) and E[xy] (X); the
// per-block loss sums go to partial[blockIdx.x].
__global__ void ssim_cols_kernel(const float *__restrict__ rows, int H, int W, const Window win,
                                 float c1, float c2, float eps, float scale,
                                 float *__restrict__ dmaps, float *__restrict__ partial) {
  __shared__ float s_sum[32];
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t P = (int64_t)H * W;
  float lsum = 0.0f;
  if (idx < 3 * P) {
    const int ch = (int)(idx / P);
    const int64_t p = idx - (int64_t)ch * P;
    const int row = (int)(p / W), col = (int)(p - (int64_t)row * W);
    float f[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    for (int d = -win.r; d <= win.r; ++d) {
      const int r2 = reflect(row + d, H);
      const float kk = win.k[d + win.r];
      for (int m = 0; m < 5; ++m)
        f[m] = fmaf(kk, rows[((int64_t)ch * 5 + m) * P + (int64_t)r2 * W + col], f[m]);
    }
    const float A = f[0], mu2 = f[1], B = f[2], Ey2 = f[3], X = f[4];
    const float s1 = B - A * A, s2 = Ey2 - mu2 * mu2, s12 = X - A * mu2;
    const float n1 = 2.0f * A * mu2 + c1, n2 = 2.0f * s12 + c2;
    const float d1 = A * A + mu2 * mu2 + c1, d2 = s1 + s2 + c2;
    const float num = n1 * n2, den = d1 * d2 + eps;
    const float S = num / den;
    const float l = (1.0f - S) * 0.5f;
    const bool inside = l > 0.0f && l < 1.0f;  // clamp(., 0, 1) passes the gradient only inside
    lsum = fminf(fmaxf(l, 0.0f), 1.0f);
    float gA = 0.0f, gB = 0.0f, gX = 0.0f;
    if (inside) {
      const float gS = -0.5f * scale;  // d(mean loss)/dS for this element
      const float dnum_dA = 2.0f * mu2 * n2 - 2.0f * mu2 * n1;
      const float dnum_dX = 2.0f * n1;
      const float dden_dA = 2.0f * A * d2 - 2.0f * A * d1;
      const float dden_dB = d1;
      const float inv = 1.0f / den;
      gA = gS * (dnum_dA - S * dden_dA) * inv;
      gB = gS * (-S * dden_dB) * inv;
      gX = gS * dnum_dX * inv;
    }
    dmaps[((int64_t)ch * 3 + 0) * P + p] = gA;
    dmaps[((int64_t)ch * 3 + 1) * P + p] = gB;
    dmaps[((int64_t)ch * 3 + 2) * P + p] = gX;
  }
  // block sum of the loss terms
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if (lane == 0) s_sum[warp] = lsum;
  __syncthreads();
  if (threadIdx.x == 0) {
    float tsum = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tsum += s_sum[w];
    partial[blockIdx.x] = tsum;
  }
}

// Adjoint of the reflected 1D filter at position j of a line of n samples
// (g at stride `step` from `base`): sum over (i, d) with reflect(i + d) == j.
__device__ __forceinline__ float adjoint_1d(const float *__restrict__ g, int64_t base,
                                            int64_t step, int j, int n, const Window &win) {
  float acc = 0.0f;
  for (int d = -win.r; d <= win.r; ++d) {
    const float kk = win.k[d + win.r];
    const int i0 = j - d;  // direct: i + d = j
    if (i0 >= 0 && i0 < n) acc = fmaf(kk, g[base + step * i0], acc);
    if (j >= 1) {  // i + d = -j < 0 reflects onto j
      const int i1 = -j - d;
      if (i1 >= 0 && i1 < n) acc = fmaf(kk, g[base + step * i1], acc);
    }
    if (j <= n - 2) {  // i + d = 2(n-1) - j > n-1 reflects onto j
      const int i2 = 2 * (n - 1) - j - d;
      if (i2 >= 0 && i2 < n) acc = fmaf(kk, g[base + step * i2], acc);
    }
  }
  return acc;
}

// Column adjoint of the three derivative maps (in place into tmp).
__global__ void ssim_cols_adj_kernel(const float *__restrict__ dmaps, int H, int W,
                                     const Window win, float *__restrict__ tmp) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t P = (int64_t)H * W;
  if (idx >= 9 * P) return;
  const int m = (int)(idx / P);  // ch * 3 + map
  const int64_t p = idx - (int64_t)m * P;
  const int row = (int)(p / W), col = (int)(p - (int64_t)row * W);
  tmp[idx] = adjoint_1d(dmaps, (int64_t)m * P + col, W, row, H, win);
}

// Row adjoint, then d(loss)/d(out) = adjA + 2 x adjB + y adjX plus the base
// loss term.  grad_out (HWC) is overwritten.
__global__ void ssim_rows_adj_kernel(const float *__restrict__ tmp, const float *__restrict__ x,
                                     const float *__restrict__ y, int H, int W, const Window win,
                                     float base_w, int l2, float *__restrict__ grad_out,
                                     float *__restrict__ partial_base) {
  __shared__ float s_sum[32];
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t P = (int64_t)H * W;
  float bsum = 0.0f;
  if (idx < 3 * P) {
    const int64_t p = idx / 3;
    const int ch = (int)(idx - p * 3);
    const int row = (int)(p / W), col = (int)(p - (int64_t)row * W);
    const int64_t rowbase = (int64_t)row * W;
    const float aA = adjoint_1d(tmp, ((int64_t)ch * 3 + 0) * P + rowbase, 1, col, W, win);
    const float aB = adjoint_1d(tmp, ((int64_t)ch * 3 + 1) * P + rowbase, 1, col, W, win);
    const float aX = adjoint_1d(tmp, ((int64_t)ch * 3 + 2) * P + rowbase, 1, col, W, win);
    const float xv = x[idx], yv = y[idx];
    float g = aA + 2.0f * xv * aB + yv * aX;
    const float diff = xv - yv;
    if (l2) {
      g = fmaf(base_w * 2.0f, diff, g);
      bsum = diff * diff;
    } else {
      const float sgn = diff > 0.0f ? 1.0f : (diff < 0.0f ? -1.0f : 0.0f);
      g = fmaf(base_w, sgn, g);
      bsum = fabsf(diff);
    }
    grad_out[idx] = g;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) bsum += __shfl_xor_sync(0xffffffffu, bsum, o);
  if (lane == 0) s_sum[warp] = bsum;
  __syncthreads();
  if (threadIdx.x == 0) {
    float tsum = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tsum += s_sum[w];
    partial_base[blockIdx.x] = tsum;
  }
}

__global__ void adam_kernel(const gsx_adam_group *__restrict__ groups, int n_groups,
                            int64_t total, const int64_t *__restrict__ offsets) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  int lo = 0, hi = n_groups - 1;  // the group holding element i
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (offsets[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  const gsx_adam_group &G = groups[lo];
  const int64_t e = i - offsets[lo];
  const float g = G.grad[e];
  float m = G.exp_avg[e], v = G.exp_avg_sq[e];
  m = m + (1.0f - G.beta1) * (g - m);  // torch: exp_avg.lerp_(grad, 1 - beta1)
  v = v * G.beta2 + (1.0f - G.beta2) * (g * g);
  G.exp_avg[e] = m;
  G.exp_avg_sq[e] = v;
  const float denom = sqrtf(v) / G.bias_correction2_sqrt + G.eps;
  G.param[e] = G.param[e] - G.step_size * (m / denom);
}

inline unsigned blocks(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace

size_t loss_workspace_bytes(int H, int W) {
  const size_t P = (size_t)H * W;
  const size_t nb = (3 * P + 255) / 256;
  return (15 * P + 9 * P + 9 * P + 2 * nb) * sizeof(float);
}

int run_ssim_loss(const float *out, const float *gt, int H, int W, int win_size, float ssim_mult,
                  int l2, float *grad_out, float *partial_out, void *ws, cudaStream_t s) {
  Window win;
  win.r = win_size / 2;
  {
    double sum = 0.0, k[kMaxWin];
    for (int i = 0; i < win_size; ++i) {
      const double xx = i - win.r;
      k[i] = exp(-xx * xx / (2.0 * 1.5 * 1.5));
      sum += k[i];
    }
    for (int i = 0; i < win_size; ++i) win.k[i] = (float)(k[i] / sum);
  }
  const int64_t P = (int64_t)H * W;
  float *rows = static_cast<float *>(ws);
  float *dmaps = rows + 15 * P;
  float *tmp = dmaps + 9 * P;
  const unsigned nb = blocks(3 * P);
  float *part_ssim = tmp + 9 * P;
  float *part_base = part_ssim + nb;
  const float scale = 1.0f / (float)(3 * P);
  count_launches(4);
  ssim_rows_kernel<<<nb, 256, 0, s>>>(out, gt, H, W, win, rows);
  ssim_cols_kernel<<<nb, 256, 0, s>>>(rows, H, W, win, 1e-4f, 9e-4f, 1e-12f, ssim_mult * scale,
                                      dmaps, part_ssim);
  ssim_cols_adj_kernel<<<blocks(9 * P), 256, 0, s>>>(dmaps, H, W, win, tmp);
  ssim_rows_adj_kernel<<<nb, 256, 0, s>>>(tmp, out, gt, H, W, win, (1.0f - ssim_mult) * scale,
                                          l2, grad_out, part_base);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "ssim loss kernels");
  if (partial_out) {
    e = cudaMemcpyAsync(partial_out, part_ssim, 2 * (size_t)nb * sizeof(float),
                        cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_status(e, "copy loss partial sums");
  }
  return GSX_OK;
}

int launch_adam(const gsx_adam_group *groups_dev, int n_groups, int64_t total,
                const int64_t *offsets_dev, cudaStream_t s) {
  if (total == 0) return GSX_OK;
  count_launches(1);
  adam_kernel<<<blocks(total), 256, 0, s>>>(groups_dev, n_groups, total, offsets_dev);
  return cuda_status(cudaGetLastError(), "adam_kernel launch");
}

}  // namespace gsx
