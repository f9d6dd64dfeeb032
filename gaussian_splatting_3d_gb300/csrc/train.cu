// train.cu -- the training step around the renderer: the photometric loss
// and its image gradient (kernels in loss_kernels.cuh), and the Adam update
// of the parameter arrays.
//
// Loss (utils/loss.py:5-24): L = m * SSIM_loss(out, gt) + (1 - m) * base(out,
// gt), base = L1 or L2 (mean), SSIM_loss = mean(clamp((1 - SSIM) / 2, 0, 1))
// over channels and pixels, with the SSIM of the kornia 0.6 series (the one
// the reference's imports fit: kornia.metrics.ssim / kornia.losses.ssim_loss):
// an 11x11 (any odd size; even sizes are rejected) normalised Gaussian window
// of sigma 1.5 applied per channel with reflected borders ("same" size),
// C1 = 0.01^2, C2 = 0.03^2,
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
#include "loss_kernels.cuh"

namespace gsx {

namespace {

// Adam: the blocks are dealt to the groups in table order, group g taking
// ceil(n_g / kAdamChunk) of them; warp 0 of each block finds its group with
// a warp scan over the groups' block counts.  Each thread updates four
// consecutive elements, with 16-byte accesses when the group's four arrays
// are 16-byte aligned.
constexpr int kAdamThreads = 256;
constexpr int kAdamVec = 4;
constexpr int kAdamChunk = kAdamThreads * kAdamVec;

__device__ __forceinline__ void adam_update(const gsx_adam_group &G, float &p, float g, float &m,
                                            float &v) {
  m = m + (1.0f - G.beta1) * (g - m);  // torch: exp_avg.lerp_(grad, 1 - beta1)
  v = v * G.beta2 + (1.0f - G.beta2) * (g * g);
  const float denom = sqrtf(v) / G.bias_correction2_sqrt + G.eps;
  p = p - G.step_size * (m / denom);
}

__global__ void __launch_bounds__(kAdamThreads)
    adam_kernel(const gsx_adam_group *__restrict__ groups, int n_groups) {
  __shared__ int s_group;
  __shared__ int64_t s_first;
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    int64_t b = blockIdx.x;  // block index still to place
    int found = n_groups;
    for (int base = 0; base < n_groups && found == n_groups; base += 32) {
      const int gi = base + lane;
      const int64_t nb = gi < n_groups ? (groups[gi].n + kAdamChunk - 1) / kAdamChunk : 0;
      int64_t inc = nb;  // inclusive scan of the block counts over the lanes
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
      }
      const unsigned hit = __ballot_sync(0xffffffffu, gi < n_groups && b < inc);
      if (hit) {
        const int l = __ffs(hit) - 1;
        const int64_t before = __shfl_sync(0xffffffffu, inc - nb, l);
        found = base + l;
        b -= before;
      } else {
        b -= __shfl_sync(0xffffffffu, inc, 31);
      }
    }
    if (lane == 0) {
      s_group = found;
      s_first = b * kAdamChunk;
    }
  }
  __syncthreads();
  if (s_group >= n_groups) return;  // the grid's spare blocks
  const gsx_adam_group G = groups[s_group];
  const int64_t e0 = s_first + (int64_t)threadIdx.x * kAdamVec;
  if (e0 >= G.n) return;
  const uintptr_t al = reinterpret_cast<uintptr_t>(G.param) | reinterpret_cast<uintptr_t>(G.grad) |
                       reinterpret_cast<uintptr_t>(G.exp_avg) |
                       reinterpret_cast<uintptr_t>(G.exp_avg_sq);
  if (e0 + kAdamVec <= G.n && (al & 15) == 0) {
    float4 p = *reinterpret_cast<const float4 *>(G.param + e0);
    const float4 g = *reinterpret_cast<const float4 *>(G.grad + e0);
    float4 m = *reinterpret_cast<const float4 *>(G.exp_avg + e0);
    float4 v = *reinterpret_cast<const float4 *>(G.exp_avg_sq + e0);
    adam_update(G, p.x, g.x, m.x, v.x);
    adam_update(G, p.y, g.y, m.y, v.y);
    adam_update(G, p.z, g.z, m.z, v.z);
    adam_update(G, p.w, g.w, m.w, v.w);
    *reinterpret_cast<float4 *>(G.exp_avg + e0) = m;
    *reinterpret_cast<float4 *>(G.exp_avg_sq + e0) = v;
    *reinterpret_cast<float4 *>(G.param + e0) = p;
  } else {
    for (int k = 0; k < kAdamVec && e0 + k < G.n; ++k) {
      const int64_t e = e0 + k;
      float p = G.param[e], m = G.exp_avg[e], v = G.exp_avg_sq[e];
      adam_update(G, p, G.grad[e], m, v);
      G.exp_avg[e] = m;
      G.exp_avg_sq[e] = v;
      G.param[e] = p;
    }
  }
}

}  // namespace

size_t loss_workspace_bytes(int H, int W) { return 9 * (size_t)H * W * sizeof(float); }

int run_ssim_loss(const float *out, const float *gt, int H, int W, int win_size, float ssim_mult,
                  int l2, float *grad_out, float *partials, void *ws, cudaStream_t s) {
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
  const int64_t nb = (3 * P + 255) / 256;  // the partial-sum slots of the C ABI
  if (partials) {
    cudaError_t e = cudaMemsetAsync(partials, 0, 2 * (size_t)nb * sizeof(float), s);
    if (e != cudaSuccess) return cuda_status(e, "clear loss partial sums");
  }
  const float scale = 1.0f / (float)(3 * P);
  const float ssim_w = ssim_mult * scale, base_w = (1.0f - ssim_mult) * scale;
  float *gmaps = static_cast<float *>(ws);
  switch (win.r) {
#define GSX_LOSS_R(RR) \
  case RR:             \
    return launch_loss<RR>(out, gt, H, W, win, ssim_w, base_w, l2, grad_out, partials, nb, gmaps, s);
    GSX_LOSS_R(0) GSX_LOSS_R(1) GSX_LOSS_R(2) GSX_LOSS_R(3) GSX_LOSS_R(4) GSX_LOSS_R(5)
    GSX_LOSS_R(6) GSX_LOSS_R(7)
#undef GSX_LOSS_R
    case 8: case 9: case 10: case 11:
      return launch_loss_r8_11(win.r, out, gt, H, W, win, ssim_w, base_w, l2, grad_out, partials, nb,
                               gmaps, s);
    case 12: case 13: case 14: case 15:
      return launch_loss_r12_15(win.r, out, gt, H, W, win, ssim_w, base_w, l2, grad_out, partials, nb,
                                gmaps, s);
    default:
      set_error("win_size %d outside 1..31", win_size);
      return GSX_ERR_INVALID_ARG;
  }
}

int launch_adam(const gsx_adam_group *groups_dev, int n_groups, int64_t total,
                const int64_t *offsets_dev, cudaStream_t s) {
  (void)offsets_dev;  // the kernel places its blocks from the groups' sizes
  if (total == 0) return GSX_OK;
  // sum over groups of ceil(n_g / chunk) <= total / chunk + n_groups
  const int64_t grid = (total + kAdamChunk - 1) / kAdamChunk + n_groups;
  if (grid > 0x7fffffffLL) {
    set_error("adam: %lld elements exceed one launch", (long long)total);
    return GSX_ERR_CAPACITY;
  }
  count_launches(1);
  adam_kernel<<<(unsigned)grid, kAdamThreads, 0, s>>>(groups_dev, n_groups);
  return cuda_status(cudaGetLastError(), "adam_kernel launch");
}

}  // namespace gsx
