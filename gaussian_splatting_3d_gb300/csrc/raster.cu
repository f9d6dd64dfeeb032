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
// GB300 layout: one CTA per tile, one thread per pixel.  Each batch of the
// tile's sorted list is gathered once into shared memory (ids, mean, cov,
// clamped alpha, SH rows padded to float4) and read by all threads as
// broadcasts.  The CTA leaves the list as soon as every pixel has saturated
// (__syncthreads_and on the per-pixel stop flag), which does not change any
// pixel: a stopped pixel takes no further Gaussians in the reference either.
// The backward reduces the per-pair gradients of a warp with a butterfly
// reduce-scatter (one shuffle per value instead of five), folds the warps
// together with shared-memory atomics, and issues one global atomic per
// (tile, Gaussian, value).
#include "gsx_internal.cuh"

namespace gsx {

namespace {

constexpr unsigned kFull = 0xffffffffu;

template <int C>
struct Sh {
  static constexpr int CC = C * C;
  static constexpr int CCP = (CC + 3) & ~3;  // per-channel smem stride
  static constexpr int GSH = 3 * CCP;        // smem floats per Gaussian
};

template <int C>
__device__ __forceinline__ void sh_basis(const float *__restrict__ c2w, float px,
                                         float py, float *Y) {
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

// sum_k sh[k] * Y[k] as the reference's fused multiply-add chain.
template <int C>
__device__ __forceinline__ float sh_dot(const float *__restrict__ s, const float *Y) {
  constexpr int CC = C * C;
  float acc = 0.0f;
  if constexpr (CC % 4 == 0) {
#pragma unroll
    for (int k = 0; k < CC; k += 4) {
      float4 q = *reinterpret_cast<const float4 *>(s + k);
      acc = fmaf(q.x, Y[k], acc);
      acc = fmaf(q.y, Y[k + 1], acc);
      acc = fmaf(q.z, Y[k + 2], acc);
      acc = fmaf(q.w, Y[k + 3], acc);
    }
  } else {
#pragma unroll
    for (int k = 0; k < CC; ++k) acc = fmaf(s[k], Y[k], acc);
  }
  return acc;
}

// radial distance of gs/src/include/kernels.h:172-187 (before the exp).
__device__ __forceinline__ float radial_of(float4 cv, float2 m, float px, float py) {
  float det = fmaf(cv.x, cv.w, -(cv.y * cv.z));
  float x = px - m.x, y = py - m.y;
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

// Length of a tile's list; 0 for empty tiles (start == -1, as the reference
// marks them) and for ranges that do not fit in [0, n_keys).
__device__ __forceinline__ int tile_list_length(const RasterArgs &a, int tile, int s0) {
  if (s0 < 0) return 0;
  const int e = a.end[tile];
  if (e < s0 || (int64_t)e > a.n_keys) return 0;
  return e - s0;
}

struct SmemLayout {
  float4 *cov;
  float2 *mean;
  float *alpha;
  int *ids;
  float *sh;
};

template <int C>
__device__ __forceinline__ SmemLayout carve(float *smem, int B) {
  SmemLayout L;
  L.cov = reinterpret_cast<float4 *>(smem);
  L.mean = reinterpret_cast<float2 *>(smem + 4 * B);
  L.alpha = smem + 6 * B;
  L.ids = reinterpret_cast<int *>(smem + 7 * B);
  L.sh = smem + 8 * B;  // 32*B bytes from the base: float4 aligned
  return L;
}

// Gather one batch of the tile's list into shared memory.
template <int C>
__device__ __forceinline__ void load_batch(const RasterArgs &a, const SmemLayout &L,
                                           int first, int nb, int t, int nthr) {
  constexpr int CC = Sh<C>::CC, CCP = Sh<C>::CCP, GSH = Sh<C>::GSH;
  for (int j = t; j < nb; j += nthr) {
    const int id = a.ids[first + j];
    if (id >= 0 && id < a.n) {
      L.ids[j] = id;
      const float *m = a.mean2d + 2 * (int64_t)id;
      const float *cv = a.cov2d + 4 * (int64_t)id;
      L.mean[j] = make_float2(m[0], m[1]);
      L.cov[j] = make_float4(cv[0], cv[1], cv[2], cv[3]);
      L.alpha[j] = fminf(a.alpha[id], 0.99f);
    } else {
      // an id outside [0, n): a transparent Gaussian far off screen, skipped
      // by every pixel (radial = inf), and no reads of the caller's arrays
      L.ids[j] = -1;
      L.mean[j] = make_float2(3.0e38f, 3.0e38f);
      L.cov[j] = make_float4(1.0f, 0.0f, 0.0f, 1.0f);
      L.alpha[j] = 0.0f;
    }
  }
  __syncthreads();
  const int total = nb * 3 * CC;
  for (int f = t; f < total; f += nthr) {
    int j = f / (3 * CC);
    int rem = f - j * (3 * CC);
    int ch = rem / CC;
    int k = rem - ch * CC;
    const int id = L.ids[j];
    L.sh[j * GSH + ch * CCP + k] = id >= 0 ? a.sh[((int64_t)id * 3 + ch) * a.sh_stride + k] : 0.0f;
  }
  __syncthreads();
}

template <int C, int MAXT>
__global__ void __launch_bounds__(MAXT) raster_forward_kernel(const RasterArgs a) {
  constexpr int CC = Sh<C>::CC, GSH = Sh<C>::GSH;
  extern __shared__ float4 smem4[];
  const int nthr = blockDim.x;
  const int B = nthr;
  SmemLayout L = carve<C>(reinterpret_cast<float *>(smem4), B);

  const int tile = blockIdx.x;
  const int t = threadIdx.x;
  const int gx = (tile % a.n_tiles_w) * a.tile_w + t % a.tile_w;
  const int gy = (tile / a.n_tiles_w) * a.tile_h + t / a.tile_w;
  const bool inside = t < a.tile_w * a.tile_h && gx < a.width && gy < a.height;
  const int s0 = a.start[tile];
  const int n = tile_list_length(a, tile, s0);
  if (n <= 0) {
    if (a.write_empty && inside) {
      float *dst = a.out + 3 * ((int64_t)gy * a.width + gx);
      dst[0] = 0.0f;
      dst[1] = 0.0f;
      dst[2] = 0.0f;
    }
    return;
  }
  const float px = fmaf((float)gx, a.psx, a.topleft[0]);
  const float py = fmaf((float)gy, a.psy, a.topleft[1]);
  float Y[CC];
  sh_basis<C>(a.c2w, px, py, Y);
  float o0 = 0.0f, o1 = 0.0f, o2 = 0.0f, T = 1.0f;
  const float thr = a.T_thresh;
  bool done = !inside;

  for (int base = 0; base < n; base += B) {
    if (__syncthreads_and(done)) break;
    const int nb = min(B, n - base);
    load_batch<C>(a, L, s0 + base, nb, t, nthr);
    if (!done) {
      for (int i = 0; i < nb; ++i) {
        if (T < thr) {
          done = true;
          break;
        }
        const float al = L.alpha[i];
        const float radial = radial_of(L.cov[i], L.mean[i], px, py);
        if (surely_skipped(radial, al)) continue;
        const float G = gsx_expf(-0.5f * radial);
        float coeff = al * T;
        coeff = coeff * G;
        if (al * G < kMinRenderAlpha) continue;
        if (isnan(coeff)) coeff = 0.0f;
        const float *s = L.sh + i * GSH;
        float y0 = gsx_sigmoidf(sh_dot<C>(s, Y));
        float y1 = gsx_sigmoidf(sh_dot<C>(s + Sh<C>::CCP, Y));
        float y2 = gsx_sigmoidf(sh_dot<C>(s + 2 * Sh<C>::CCP, Y));
        if (isnan(y0 * coeff)) y0 = 0.0f;
        if (isnan(y1 * coeff)) y1 = 0.0f;
        if (isnan(y2 * coeff)) y2 = 0.0f;
        o0 = fmaf(coeff, y0, o0);
        o1 = fmaf(coeff, y1, o1);
        o2 = fmaf(coeff, y2, o2);
        T = T * fmaf(-al, G, 1.0f);
      }
      if (T < thr) done = true;
    }
  }
  if (inside) {
    float *dst = a.out + 3 * ((int64_t)gy * a.width + gx);
    dst[0] = o0;
    dst[1] = o1;
    dst[2] = o2;
  }
}

// Butterfly reduce-scatter of V = 32*R values over a warp: afterwards lane l
// holds the warp sums of value indices l*R .. l*R + R - 1 in v[0..R-1].
template <int V>
__device__ __forceinline__ void warp_reduce_scatter(float (&v)[V], int lane) {
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int o = 16 >> s;
    const int half = (V >> s) / 2;
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int k = 0; k < half; ++k) {
      float send = up ? v[k] : v[k + half];
      float keep = up ? v[k + half] : v[k];
      v[k] = keep + __shfl_xor_sync(kFull, send, o);
    }
  }
}

template <int C, int MAXT>
__global__ void __launch_bounds__(MAXT) raster_backward_kernel(const RasterArgs a, int B) {
  constexpr int CC = Sh<C>::CC, CCP = Sh<C>::CCP, GSH = Sh<C>::GSH;
  constexpr int NV = 6 + 3 * CC;  // gm0 gm1 gc0 gc12 gc3 galpha gsh[3*CC]
  constexpr int V = ((NV + 31) / 32) * 32;
  constexpr int R = V / 32;
  extern __shared__ float4 smem4[];
  float *smem = reinterpret_cast<float *>(smem4);
  SmemLayout L = carve<C>(smem, B);
  float *s_grad = L.sh + B * GSH;               // [B][NV]
  int *s_touched = reinterpret_cast<int *>(s_grad + B * NV);

  const int nthr = blockDim.x;
  const int tile = blockIdx.x;
  const int t = threadIdx.x, lane = t & 31;
  const int gx = (tile % a.n_tiles_w) * a.tile_w + t % a.tile_w;
  const int gy = (tile / a.n_tiles_w) * a.tile_h + t / a.tile_w;
  const bool inside = t < a.tile_w * a.tile_h && gx < a.width && gy < a.height;
  const int s0 = a.start[tile];
  const int n = tile_list_length(a, tile, s0);
  if (n <= 0) return;
  const float px = fmaf((float)gx, a.psx, a.topleft[0]);
  const float py = fmaf((float)gy, a.psy, a.topleft[1]);
  float Y[CC];
  sh_basis<C>(a.c2w, px, py, Y);
  float fin[3] = {0.0f, 0.0f, 0.0f}, go[3] = {0.0f, 0.0f, 0.0f};
  if (inside) {
    const int64_t pix = 3 * ((int64_t)gy * a.width + gx);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      fin[ch] = a.final_img[pix + ch];
      go[ch] = a.grad_out[pix + ch];
    }
  }
  float o[3] = {0.0f, 0.0f, 0.0f};
  float T = 1.0f;
  const float thr = a.T_thresh;
  bool done = !inside;

  for (int base = 0; base < n; base += B) {
    if (__syncthreads_and(done)) break;
    const int nb = min(B, n - base);
    for (int f = t; f < nb * NV; f += nthr) s_grad[f] = 0.0f;
    for (int j = t; j < nb; j += nthr) s_touched[j] = 0;
    load_batch<C>(a, L, s0 + base, nb, t, nthr);

    for (int i = 0; i < nb; ++i) {
      if (__all_sync(kFull, done)) break;
      bool contrib = false;
      float v[V];
#pragma unroll
      for (int k = 0; k < V; ++k) v[k] = 0.0f;
      if (!done) {
        if (T < thr) {
          done = true;
        } else {
          const float al = L.alpha[i];
          const float4 cv = L.cov[i];
          const float2 m = L.mean[i];
          const float radial = radial_of(cv, m, px, py);
          if (!surely_skipped(radial, al)) {
            const float G = gsx_expf(-0.5f * radial);
            if (!(al * G < kMinRenderAlpha)) {
              contrib = true;
              float coeff = al * T * G;
              if (isnan(coeff)) coeff = 0.0f;
              const float *s = L.sh + i * GSH;
              float y[3];
#pragma unroll
              for (int ch = 0; ch < 3; ++ch) {
                y[ch] = gsx_sigmoidf(sh_dot<C>(s + ch * CCP, Y));
                if (isnan(y[ch] * coeff)) y[ch] = 0.0f;
                o[ch] = fmaf(coeff, y[ch], o[ch]);
              }
#pragma unroll
              for (int ch = 0; ch < 3; ++ch) {
                const float w = coeff * (y[ch] * (1.0f - y[ch])) * go[ch];
#pragma unroll
                for (int k = 0; k < CC; ++k) v[6 + ch * CC + k] = w * Y[k];
              }
              const float one_m = fmaf(-al, G, 1.0f);
              float P = 0.0f;
#pragma unroll
              for (int ch = 0; ch < 3; ++ch) {
                const float q = (fin[ch] - o[ch]) / one_m;
                P = fmaf(go[ch], fmaf(y[ch], T, -q), P);
              }
              const float dg = P * al * G;
              const float det = fmaf(cv.x, cv.w, -(cv.y * cv.z));
              const float x = px - m.x, yy = py - m.y;
              const float tmpx = fmaf(x, cv.w, -(yy * cv.z)) / det;
              const float tmpy = fmaf(-x, cv.y, yy * cv.x) / det;
              const float dx = dg * tmpx, dy = dg * tmpy;
              v[0] = dx;
              v[1] = dy;
              v[2] = 0.5f * (dx * tmpx);
              v[3] = 0.5f * (dx * tmpy);
              v[4] = 0.5f * (dy * tmpy);
              v[5] = P * G;
              T = T * one_m;
            }
          }
        }
      }
      if (__ballot_sync(kFull, contrib)) {
        warp_reduce_scatter<V>(v, lane);
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int idx = lane * R + r;
          if (idx < NV && v[r] != 0.0f) atomicAdd(&s_grad[i * NV + idx], v[r]);
        }
        if (lane == 0) s_touched[i] = 1;
      }
    }
    if (!done && T < thr) done = true;
    __syncthreads();
    for (int f = t; f < nb * NV; f += nthr) {
      const int j = f / NV, idx = f - j * NV;
      if (!s_touched[j] || L.ids[j] < 0) continue;
      const float val = s_grad[f];
      if (val == 0.0f) continue;
      const int64_t id = L.ids[j];
      if (idx < 2) {
        atomicAdd(a.g_mean2d + 2 * id + idx, val);
      } else if (idx == 2) {
        atomicAdd(a.g_cov2d + 4 * id, val);
      } else if (idx == 3) {
        atomicAdd(a.g_cov2d + 4 * id + 1, val);
        atomicAdd(a.g_cov2d + 4 * id + 2, val);
      } else if (idx == 4) {
        atomicAdd(a.g_cov2d + 4 * id + 3, val);
      } else if (idx == 5) {
        atomicAdd(a.g_alpha + id, val);
      } else {
        const int e = idx - 6, ch = e / CC, k = e - ch * CC;
        atomicAdd(a.g_sh + (id * 3 + ch) * a.sh_stride + k, val);
      }
    }
  }
}

template <int C>
size_t fwd_smem(int nthr) {
  return (size_t)nthr * (8 + Sh<C>::GSH) * sizeof(float);
}

template <int C>
size_t bwd_smem(int B) {
  constexpr int NV = 6 + 3 * Sh<C>::CC;
  return (size_t)B * (8 + Sh<C>::GSH + NV + 1) * sizeof(float);
}

inline int block_threads(const RasterArgs &a) { return (a.tile_w * a.tile_h + 31) / 32 * 32; }

template <int C, int MAXT>
int launch_fwd_tt(const RasterArgs &a, cudaStream_t s) {
  const int nthr = block_threads(a);
  const size_t smem = fwd_smem<C>(nthr);
  cudaError_t e = cudaFuncSetAttribute(raster_forward_kernel<C, MAXT>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return cuda_status(e, "raster_forward smem attribute");
  const unsigned grid = (unsigned)(a.n_tiles_w * a.n_tiles_h);
  raster_forward_kernel<C, MAXT><<<grid, nthr, smem, s>>>(a);
  return cuda_status(cudaGetLastError(), "raster_forward_kernel launch");
}

template <int C>
int launch_fwd_t(const RasterArgs &a, cudaStream_t s) {
  return block_threads(a) <= 256 ? launch_fwd_tt<C, 256>(a, s) : launch_fwd_tt<C, 1024>(a, s);
}

template <int C, int MAXT>
int launch_bwd_tt(const RasterArgs &a, cudaStream_t s) {
  const int nthr = block_threads(a);
  const int B = nthr < 128 ? nthr : 128;
  const size_t smem = bwd_smem<C>(B);
  cudaError_t e = cudaFuncSetAttribute(raster_backward_kernel<C, MAXT>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return cuda_status(e, "raster_backward smem attribute");
  const unsigned grid = (unsigned)(a.n_tiles_w * a.n_tiles_h);
  raster_backward_kernel<C, MAXT><<<grid, nthr, smem, s>>>(a, B);
  return cuda_status(cudaGetLastError(), "raster_backward_kernel launch");
}

template <int C>
int launch_bwd_t(const RasterArgs &a, cudaStream_t s) {
  return block_threads(a) <= 256 ? launch_bwd_tt<C, 256>(a, s) : launch_bwd_tt<C, 1024>(a, s);
}

}  // namespace

int launch_raster_forward(const RasterArgs &a, int C, cudaStream_t s) {
  if ((int64_t)a.n_tiles_w * a.n_tiles_h == 0) return GSX_OK;
  switch (C) {
    case 1: return launch_fwd_t<1>(a, s);
    case 2: return launch_fwd_t<2>(a, s);
    case 3: return launch_fwd_t<3>(a, s);
    case 4: return launch_fwd_t<4>(a, s);
  }
  set_error("SH order C must be 1..4 (got %d)", C);
  return GSX_ERR_INVALID_ARG;
}

int launch_raster_backward(const RasterArgs &a, int C, cudaStream_t s) {
  if ((int64_t)a.n_tiles_w * a.n_tiles_h == 0) return GSX_OK;
  switch (C) {
    case 1: return launch_bwd_t<1>(a, s);
    case 2: return launch_bwd_t<2>(a, s);
    case 3: return launch_bwd_t<3>(a, s);
    case 4: return launch_bwd_t<4>(a, s);
  }
  set_error("SH order C must be 1..4 (got %d)", C);
  return GSX_ERR_INVALID_ARG;
}

}  // namespace gsx
