// loss_r8.cu -- the photometric loss's kernels for window radii 8..11
// (windows 17..23), in their own translation unit so they compile in parallel
// with train.cu's radii 0..7.
#include "loss_kernels.cuh"

namespace gsx {

int launch_loss_r8_11(int R, const float *out, const float *gt, int H, int W, const Window &win,
                      float ssim_w, float base_w, int l2, float *grad_out, float *partials,
                      int64_t nb, float *gmaps, cudaStream_t s) {
  switch (R) {
    case 8:
      return launch_loss<8>(out, gt, H, W, win, ssim_w, base_w, l2, grad_out, partials, nb, gmaps, s);
    case 9:
      return launch_loss<9>(out, gt, H, W, win, ssim_w, base_w, l2, grad_out, partials, nb, gmaps, s);
    case 10:
      return launch_loss<10>(out, gt, H, W, win, ssim_w, base_w, l2, grad_out, partials, nb, gmaps, s);
    case 11:
      return launch_loss<11>(out, gt, H, W, win, ssim_w, base_w, l2, grad_out, partials, nb, gmaps, s);
    default:
      set_error("window radius %d outside 8..11", R);
      return GSX_ERR_INVALID_ARG;
  }
}

}  // namespace gsx
