// loss_kernels.cuh -- the photometric loss's tiled kernels (ssim_fwd_kernel,
// ssim_adj_kernel) and their launcher, templated on the window radius R.
// train.cu instantiates R = 0..7, loss_r8.cu R = 8..11 and loss_r12.cu
// R = 12..15, so that the radii compile in parallel.
#pragma once

#include "gsx_internal.cuh"

namespace gsx {

constexpr int kMaxWin = 31;

struct Window {
  float k[kMaxWin];
  int r;  // radius: window = 2r + 1
};

// The loss passes for window radii 8..11 and 12..15 (loss_r8.cu,
// loss_r12.cu); same arguments as launch_loss<R>.
int launch_loss_r8_11(int R, const float *out, const float *gt, int H, int W, const Window &win,
                      float ssim_w, float base_w, int l2, float *grad_out, float *partials,
                      int64_t nb, float *gmaps, cudaStream_t s);
int launch_loss_r12_15(int R, const float *out, const float *gt, int H, int W, const Window &win,
                       float ssim_w, float base_w, int l2, float *grad_out, float *partials,
                       int64_t nb, float *gmaps, cudaStream_t s);

namespace {

// kornia's reflected border (no edge repeat) for m in [-(n-1), 2(n-1)].
__device__ __forceinline__ int reflect(int m, int n) {
  if (m < 0) return -m;
  if (m > n - 1) return 2 * (n - 1) - m;
  return m;
}

// The loss runs as two tiled passes over 32x32 pixel tiles, one channel at a
// time, each stage in shared memory:
//   ssim_fwd_kernel: x = out, y = gt over the tile plus a halo of R with
//     reflected indices -> the window's horizontal pass of the five maps x,
//     y, x^2, y^2, xy -> the vertical pass -> SSIM and the derivatives of the
//     clamped per-element loss with respect to the filtered maps mu1 (A),
//     E[x^2] (B) and E[xy] (X), written as planar maps [3 ch][3][H][W], and
//     the CTA's sum of loss terms;
//   ssim_adj_kernel: the three derivative maps over the tile plus a halo of
//     R -> the filter's adjoint, vertical then horizontal (the reflection
//     folded back onto the border pixels, exactly the transpose of the
//     forward's reflected filter) -> dL/dout = adjA + 2 x adjB + y adjX plus
//     the L1/L2 term, all three channels of a pixel written together.
// A CTA walks tiles blockIdx.x, blockIdx.x + gridDim.x, ... so its loss
// sums land in partial[blockIdx.x] in a fixed order (deterministic).
constexpr int kLT = 32;          // tile edge (pixels)
constexpr int kLossThreads = 256;
constexpr int kRowsPerThread = kLT / (kLossThreads / 32);  // 4: a warp per 4 rows, a lane per column

__device__ __forceinline__ float block_sum(float v, float *s_sum) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) s_sum[warp] = v;
  __syncthreads();
  float t = 0.0f;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_sum[w];
  return t;
}

template <int R>
__global__ void __launch_bounds__(kLossThreads)
    ssim_fwd_kernel(const float *__restrict__ x, const float *__restrict__ y, int H, int W,
                    const Window win, float c1, float c2, float eps, int tiles_x, int n_tiles,
                    float *__restrict__ gmaps, float *__restrict__ partial) {
  constexpr int EX = kLT + 2 * R, EY = kLT + 2 * R;
  extern __shared__ float sm[];
  __shared__ float s_sum[32];
  float *in_x = sm, *in_y = in_x + EX * EY;
  float *hm = in_y + EX * EY;  // [5][EY][kLT]
  const int64_t P = (int64_t)H * W;
  const int t = threadIdx.x, col = t & 31, rb = (t >> 5) * kRowsPerThread;
  float lsum = 0.0f;
  for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int ty0 = (tile / tiles_x) * kLT, tx0 = (tile % tiles_x) * kLT;
    for (int c = 0; c < 3; ++c) {
      __syncthreads();  // the previous pass's reads of shared memory are done
      for (int f = t; f < EX * EY; f += kLossThreads) {
        const int ry = f / EX, rx = f - ry * EX;
        const int ay = ty0 - R + ry, ax = tx0 - R + rx;
        float vx = 0.0f, vy = 0.0f;
        if (ay <= H - 1 + R && ax <= W - 1 + R) {  // feeds an output inside the image
          const int64_t q = 3 * ((int64_t)reflect(ay, H) * W + reflect(ax, W)) + c;
          vx = x[q];
          vy = y[q];
        }
        in_x[f] = vx;
        in_y[f] = vy;
      }
      __syncthreads();
      for (int ry = t >> 5; ry < EY; ry += kLossThreads / 32) {  // horizontal pass
        const float *px = in_x + ry * EX + col, *py = in_y + ry * EX + col;
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f, a4 = 0.0f;
#pragma unroll
        for (int d = 0; d <= 2 * R; ++d) {
          const float kk = win.k[d], xv = px[d], yv = py[d];
          a0 = fmaf(kk, xv, a0);
          a1 = fmaf(kk, yv, a1);
          a2 = fmaf(kk, xv * xv, a2);
          a3 = fmaf(kk, yv * yv, a3);
          a4 = fmaf(kk, xv * yv, a4);
        }
        float *h = hm + ry * kLT + col;
        h[0 * EY * kLT] = a0;
        h[1 * EY * kLT] = a1;
        h[2 * EY * kLT] = a2;
        h[3 * EY * kLT] = a3;
        h[4 * EY * kLT] = a4;
      }
      __syncthreads();
      // vertical pass: this thread's column, rows rb .. rb+3 of the tile
      float F[5][kRowsPerThread];
#pragma unroll
      for (int m = 0; m < 5; ++m) {
#pragma unroll
        for (int o = 0; o < kRowsPerThread; ++o) F[m][o] = 0.0f;
        const float *h = hm + (m * EY + rb) * kLT + col;
#pragma unroll
        for (int s = 0; s < 2 * R + kRowsPerThread; ++s) {
          const float v = h[s * kLT];
#pragma unroll
          for (int o = 0; o < kRowsPerThread; ++o)
            if (s - o >= 0 && s - o <= 2 * R) F[m][o] = fmaf(win.k[s - o], v, F[m][o]);
        }
      }
      const int gx = tx0 + col;
#pragma unroll
      for (int o = 0; o < kRowsPerThread; ++o) {
        const int gy = ty0 + rb + o;
        if (gy >= H || gx >= W) continue;
        const float A = F[0][o], mu2 = F[1][o], B = F[2][o], Ey2 = F[3][o], X = F[4][o];
        const float s1 = B - A * A, s2 = Ey2 - mu2 * mu2, s12 = X - A * mu2;
        const float n1 = 2.0f * A * mu2 + c1, n2 = 2.0f * s12 + c2;
        const float d1 = A * A + mu2 * mu2 + c1, d2 = s1 + s2 + c2;
        const float num = n1 * n2, den = d1 * d2 + eps;
        const float S = num / den;
        const float l = (1.0f - S) * 0.5f;
        const bool inner = l > 0.0f && l < 1.0f;  // clamp(., 0, 1) passes the gradient only inside
        lsum += fminf(fmaxf(l, 0.0f), 1.0f);
        float gA = 0.0f, gB = 0.0f, gX = 0.0f;
        if (inner) {  // d l / d(A, B, X), the mean's 1/(3HW) applied by the caller's scale
          const float inv = 1.0f / den;
          const float dnum_dA = 2.0f * mu2 * n2 - 2.0f * mu2 * n1;
          const float dden_dA = 2.0f * A * d2 - 2.0f * A * d1;
          gA = -0.5f * (dnum_dA - S * dden_dA) * inv;
          gB = -0.5f * (-S * d1) * inv;
          gX = -0.5f * (2.0f * n1) * inv;
        }
        const int64_t p = (int64_t)gy * W + gx;
        gmaps[(c * 3 + 0) * P + p] = gA;
        gmaps[(c * 3 + 1) * P + p] = gB;
        gmaps[(c * 3 + 2) * P + p] = gX;
      }
    }
  }
  const float tsum = block_sum(lsum, s_sum);
  if (t == 0 && partial) partial[blockIdx.x] = tsum;
}

// Adjoint of the reflected 1D filter at output j (0 <= j < n) of a line whose
// samples g(i) sit at line[(i - i0) * step]: the sum over taps d of k[d + R]
// times g(i) for every i with reflect(i + d) == j.  The sources lie in
// [j - R, j + R] and, near a border, in [0, R) or (n - 1 - R, n - 1].
template <int R>
__device__ __forceinline__ float adjoint_border(const float *__restrict__ line, int i0, int step,
                                                int j, int n, const Window &win) {
  float acc = 0.0f;
#pragma unroll 1
  for (int d = -R; d <= R; ++d) {  // a loop, not unrolled: it runs on border tiles only
    const float kk = win.k[d + R];
    const int a = j - d;  // direct
    if (a >= 0 && a < n) acc = fmaf(kk, line[(a - i0) * step], acc);
    const int b = -j - d;  // i + d = -j reflects onto j
    if (j >= 1 && b >= 0 && b < n) acc = fmaf(kk, line[(b - i0) * step], acc);
    const int e = 2 * (n - 1) - j - d;  // i + d = 2(n-1) - j reflects onto j
    if (j <= n - 2 && e >= 0 && e < n) acc = fmaf(kk, line[(e - i0) * step], acc);
  }
  return acc;
}

template <int R>
__global__ void __launch_bounds__(kLossThreads)
    ssim_adj_kernel(const float *__restrict__ gmaps, const float *__restrict__ x,
                    const float *__restrict__ y, int H, int W, const Window win, float ssim_w,
                    float base_w, int l2, int tiles_x, int n_tiles, float *__restrict__ grad_out,
                    float *__restrict__ partial_base) {
  constexpr int EX = kLT + 2 * R, EY = kLT + 2 * R;
  extern __shared__ float sm[];
  __shared__ float s_sum[32];
  float *gs = sm;                // [3][EY][EX]
  float *av = gs + 3 * EY * EX;  // [3][kLT][EX]
  const int64_t P = (int64_t)H * W;
  const int t = threadIdx.x, col = t & 31, rb = (t >> 5) * kRowsPerThread;
  float bsum = 0.0f;
  for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int ty0 = (tile / tiles_x) * kLT, tx0 = (tile % tiles_x) * kLT;
    // every output row (column) of the tile is at least R + 1 away from both
    // image borders: the adjoint is the plain flipped filter
    const bool inner_y = ty0 >= R + 1 && ty0 + kLT <= H - 1 - R;
    const bool inner_x = tx0 >= R + 1 && tx0 + kLT <= W - 1 - R;
    float gacc[3][kRowsPerThread];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      __syncthreads();
      for (int f = t; f < 3 * EY * EX; f += kLossThreads) {
        const int m = f / (EY * EX), r = f - m * (EY * EX);
        const int ry = r / EX, rx = r - ry * EX;
        const int ay = ty0 - R + ry, ax = tx0 - R + rx;
        gs[f] = (ay >= 0 && ay < H && ax >= 0 && ax < W) ? gmaps[(c * 3 + m) * P + (int64_t)ay * W + ax]
                                                         : 0.0f;
      }
      __syncthreads();
      // vertical adjoint: rows ty0 .. ty0+31 of the region's EX columns
      for (int f = t; f < 3 * (kLT / kRowsPerThread) * EX; f += kLossThreads) {
        const int m = f / ((kLT / kRowsPerThread) * EX), r = f - m * ((kLT / kRowsPerThread) * EX);
        const int rb2 = (r / EX) * kRowsPerThread, rx = r - (r / EX) * EX;
        const float *g = gs + m * EY * EX + rx;
        float *dst = av + (m * kLT + rb2) * EX + rx;
        if (inner_y) {
          float acc[kRowsPerThread];
#pragma unroll
          for (int o = 0; o < kRowsPerThread; ++o) acc[o] = 0.0f;
#pragma unroll
          for (int s = 0; s < 2 * R + kRowsPerThread; ++s) {  // region row rb2 + s
            const float v = g[(rb2 + s) * EX];
#pragma unroll
            for (int o = 0; o < kRowsPerThread; ++o)  // output row rb2 + o, tap d = R + o - s
              if (s - o >= 0 && s - o <= 2 * R) acc[o] = fmaf(win.k[2 * R - (s - o)], v, acc[o]);
          }
#pragma unroll
          for (int o = 0; o < kRowsPerThread; ++o) dst[o * EX] = acc[o];
        } else {
#pragma unroll
          for (int o = 0; o < kRowsPerThread; ++o) {
            const int j = ty0 + rb2 + o;
            dst[o * EX] = j < H ? adjoint_border<R>(g, ty0 - R, EX, j, H, win) : 0.0f;
          }
        }
      }
      __syncthreads();
      // horizontal adjoint: this thread's column of the tile, rows rb .. rb+3,
      // then dL/dout for this channel
      const int gx = tx0 + col;
#pragma unroll
      for (int o = 0; o < kRowsPerThread; ++o) {
        float adj[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          const float *line = av + (m * kLT + rb + o) * EX;
          float acc = 0.0f;
          if (inner_x) {
#pragma unroll
            for (int d = -R; d <= R; ++d) acc = fmaf(win.k[d + R], line[col + R - d], acc);
          } else if (gx < W) {
            acc = adjoint_border<R>(line, tx0 - R, 1, gx, W, win);
          }
          adj[m] = acc;
        }
        const int gy = ty0 + rb + o;
        float g = 0.0f;
        if (gy < H && gx < W) {
          const int64_t q = 3 * ((int64_t)gy * W + gx) + c;
          const float xv = x[q], yv = y[q];
          g = ssim_w * (adj[0] + 2.0f * xv * adj[1] + yv * adj[2]);
          const float diff = xv - yv;
          if (l2) {
            g = fmaf(base_w * 2.0f, diff, g);
            bsum = fmaf(diff, diff, bsum);
          } else {
            const float sgn = diff > 0.0f ? 1.0f : (diff < 0.0f ? -1.0f : 0.0f);
            g = fmaf(base_w, sgn, g);
            bsum += fabsf(diff);
          }
        }
        gacc[c][o] = g;
      }
    }
    // the three channels of each pixel together: HWC rows stay contiguous
    const int gx = tx0 + col;
#pragma unroll
    for (int o = 0; o < kRowsPerThread; ++o) {
      const int gy = ty0 + rb + o;
      if (gy < H && gx < W) {
        float *dst = grad_out + 3 * ((int64_t)gy * W + gx);
        dst[0] = gacc[0][o];
        dst[1] = gacc[1][o];
        dst[2] = gacc[2][o];
      }
    }
  }
  const float tsum = block_sum(bsum, s_sum);
  if (t == 0 && partial_base) partial_base[blockIdx.x] = tsum;
}

template <typename K>
cudaError_t ensure_dyn_smem(K kernel, size_t smem, size_t &done) {
  if (smem <= done || smem <= 48 * 1024) return cudaSuccess;
  cudaError_t e =
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) done = smem;
  return e;
}

template <int R>
int launch_loss(const float *out, const float *gt, int H, int W, const Window &win,
                float ssim_w, float base_w, int l2, float *grad_out, float *partials,
                int64_t nb, float *gmaps, cudaStream_t s) {
  constexpr int EX = kLT + 2 * R, EY = kLT + 2 * R;
  const size_t smem1 = (size_t)(2 * EX * EY + 5 * EY * kLT) * sizeof(float);
  const size_t smem2 = (size_t)(3 * EY * EX + 3 * kLT * EX) * sizeof(float);
  static size_t done1 = 0, done2 = 0;
  cudaError_t e = ensure_dyn_smem(ssim_fwd_kernel<R>, smem1, done1);
  if (e == cudaSuccess) e = ensure_dyn_smem(ssim_adj_kernel<R>, smem2, done2);
  if (e != cudaSuccess) return cuda_status(e, "ssim kernels smem attribute");
  const int tiles_x = (W + kLT - 1) / kLT, tiles_y = (H + kLT - 1) / kLT;
  const int n_tiles = tiles_x * tiles_y;
  // one partial sum per CTA, in the caller's nb slots (nb >= 1)
  const int grid = (int)(n_tiles < nb ? n_tiles : nb);
  count_launches(2);
  ssim_fwd_kernel<R><<<grid, kLossThreads, smem1, s>>>(out, gt, H, W, win, 1e-4f, 9e-4f, 1e-12f,
                                                        tiles_x, n_tiles, gmaps, partials);
  ssim_adj_kernel<R><<<grid, kLossThreads, smem2, s>>>(gmaps, out, gt, H, W, win, ssim_w, base_w,
                                                        l2, tiles_x, n_tiles, grad_out,
                                                        partials ? partials + nb : nullptr);
  return cuda_status(cudaGetLastError(), "ssim loss kernels");
}

}  // namespace

}  // namespace gsx
