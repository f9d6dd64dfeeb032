// loss_r12.cu -- the photometric loss's kernels for window radii 12..15
// (windows 25..31), in their own translation unit so they compile in parallel
// with train.cu's radii 0..7.
#include "loss_kernels.cuh"

namespace gsx {

int launch_loss_r12_15(int R, const float *out, const float *gt, int H, int W, const Window &win,
                       float ssim_w, float base_w, int l2, float *grad_out, float *partials,
                       int64_t nb, float *gmaps, cudaStream_t s) {
  switch (R) {
    case 12:
      return launch_loss<12>(out, gt, H, W, win, ssim_w, base_w, l2, grad_out, partials, nb, gmaps, s);
    case 13:
      return launch_loss<13>(out, gt, H, W, win, ssim_w, base_w, l2, grad_out, partials, nb, gmaps, s);
    case 14:
      return launch_loss<14>(out, gt, H, W, win, ssim_w, base_w, l2, grad_out, partials, nb, gmaps, s);
    case 15:
      return launch_loss<15>(out, gt, H, W, win, ssim_w, base_w, l2, grad_out, partials, nb, gmaps, s);
    default:
      set_error("window radius %d outside 12..15", R);
      return GSX_ERR_INVALID_ARG;
  }
}

}  // namespace gsx
