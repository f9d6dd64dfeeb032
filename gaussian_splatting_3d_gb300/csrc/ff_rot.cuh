// ff_rot.cuh -- the projection backward's rotation matrix in float-float
// (host and device: the host build of the same functions is what the CPU
// test tests/test_ff_rotation_host.py checks against double precision).
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace gsx {

// ---- the backward's rotation in float-float ---------------------------------
// The quaternion gradient of a needle-like Gaussian is a small difference of
// large terms (dL/dSigma of order 1e6 against M's thin columns), so it is
// only as accurate as R: R in float (a few ulp per entry) moves dL/dq by
// ~1e-4 of the tensor's largest entry against an exact evaluation, while R
// exact to ~2^-44 and rounded once into M = R diag(s) leaves ~2e-5 (the
// other float stages' share).  R is formed as N / |q|^2 (N the quadratic form
// of the unnormalised quaternion, equal to the normalised formula) with the
// error-free transformations two-product (FMA) and two-sum (Knuth), and a
// Newton-refined reciprocal.  The forward keeps the float R of quat_rot,
// whose rounding the rendered covariance reproduces bit for bit.
struct FF {
  float hi, lo;
};

__host__ __device__ __forceinline__ FF ff_prod(float a, float b) {
  const float p = a * b;
  return {p, fmaf(a, b, -p)};
}

__host__ __device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b.hi - bb);
  const float lo = e + (a.lo + b.lo);
  const float hi = s + lo;
  return {hi, lo - (hi - s)};
}

__host__ __device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const FF p = ff_prod(a.hi, b.hi);
  const float lo = fmaf(a.hi, b.lo, a.lo * b.hi) + p.lo;
  const float hi = p.hi + lo;
  return {hi, lo - (hi - p.hi)};
}

// R(q / |q|) in float-float, written as R (rounded) and M = R diag(s) (one
// rounding of the float-float product) one entry at a time; false (nothing
// written) for |q| below the 1e-12 clamp.
__host__ __device__ __forceinline__ bool frame_ff(const float4 q, const float (&s)[3], float (&R)[3][3],
                                         float (&M)[3][3]) {
  const float w = q.x, x = q.y, y = q.z, z = q.w;
  const FF ww = ff_prod(w, w), xx = ff_prod(x, x), yy = ff_prod(y, y), zz = ff_prod(z, z);
  const FF s_ww_xx = ff_add(ww, xx), s_yy_zz = ff_add(yy, zz);
  const FF n2 = ff_add(s_ww_xx, s_yy_zz);
  if (!(n2.hi >= 1e-24f)) return false;
  const float r0 = 1.0f / n2.hi;
  const float e = fmaf(-n2.hi, r0, 1.0f) - n2.lo * r0;  // 1 - |q|^2 r0
  const FF inv = {r0, r0 * e};
  const FF inv2 = {2.0f * r0, 2.0f * (r0 * e)};  // 2 / |q|^2, exact doubling
  auto put = [&](int i, int j, FF num, const FF &scale) {
    const FF r = ff_mul(num, scale);
    R[i][j] = r.hi;
    M[i][j] = fmaf(r.hi, s[j], r.lo * s[j]);
  };
  const FF d_ww_xx = ff_add(ww, {-xx.hi, -xx.lo}), d_yy_zz = ff_add(yy, {-zz.hi, -zz.lo});
  put(0, 0, ff_add(s_ww_xx, {-s_yy_zz.hi, -s_yy_zz.lo}), inv);
  put(1, 1, ff_add(d_ww_xx, d_yy_zz), inv);
  put(2, 2, ff_add(d_ww_xx, {-d_yy_zz.hi, -d_yy_zz.lo}), inv);
  {
    const FF xy = ff_prod(x, y), wz = ff_prod(w, z);
    put(0, 1, ff_add(xy, {-wz.hi, -wz.lo}), inv2);
    put(1, 0, ff_add(xy, wz), inv2);
  }
  {
    const FF xz = ff_prod(x, z), wy = ff_prod(w, y);
    put(0, 2, ff_add(xz, wy), inv2);
    put(2, 0, ff_add(xz, {-wy.hi, -wy.lo}), inv2);
  }
  {
    const FF yz = ff_prod(y, z), wx = ff_prod(w, x);
    put(1, 2, ff_add(yz, {-wx.hi, -wx.lo}), inv2);
    put(2, 1, ff_add(yz, wx), inv2);
  }
  return true;
}

}  // namespace gsx
