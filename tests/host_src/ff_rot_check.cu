// Host build of the projection backward's float-float rotation
// (gaussian_splatting_3d_gb300/csrc/ff_rot.cuh) against a double-precision
// evaluation of R(q / |q|) and M = R diag(s), for seeded quaternions of
// several magnitudes (unit, small, large, one near-zero component).  Prints
// "max_r_err max_m_ulp m_mismatches n" on one line.
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include "ff_rot.cuh"

static uint64_t state = 0x9E3779B97F4A7C15ull;
static double uniform() {  // xorshift64*, in [-1, 1)
  state ^= state >> 12;
  state ^= state << 25;
  state ^= state >> 27;
  return (double)((state * 0x2545F4914F6CDD1Dull) >> 11) / 9007199254740992.0 * 2.0 - 1.0;
}

int main() {
  const int n = 200000;
  double max_r = 0.0, max_m_ulp = 0.0;
  long mism = 0;
  for (int it = 0; it < n; ++it) {
    const float mag = (it % 4 == 0) ? 1e-3f : (it % 4 == 1) ? 37.0f : 1.0f;
    float q[4];
    for (int k = 0; k < 4; ++k) q[k] = (float)uniform() * mag;
    if (it % 7 == 0) q[it % 4] *= 1e-6f;
    const float s[3] = {(float)exp(uniform() * 5.0), (float)exp(uniform() * 5.0), (float)exp(uniform() * 5.0)};
    float R[3][3], M[3][3];
    if (!gsx::frame_ff(make_float4(q[0], q[1], q[2], q[3]), s, R, M)) continue;
    const double nq = sqrt((double)q[0] * q[0] + (double)q[1] * q[1] + (double)q[2] * q[2] + (double)q[3] * q[3]);
    const double w = q[0] / nq, x = q[1] / nq, y = q[2] / nq, z = q[3] / nq;
    const double Rd[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)},
                             {2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)},
                             {2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)}};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        const double er = fabs((double)R[i][j] - Rd[i][j]);
        if (er > max_r) max_r = er;
        const double md = Rd[i][j] * (double)s[j];
        const float mr = (float)md;  // correctly rounded M
        if (mr != M[i][j]) ++mism;
        const double ulp = fabs(md) > 0 ? fabs((double)M[i][j] - md) / (nextafterf(fabsf(mr), INFINITY) - fabsf(mr)) : 0;
        if (ulp > max_m_ulp) max_m_ulp = ulp;
      }
  }
  printf("%.3e %.3f %ld %d\n", max_r, max_m_ulp, mism, n);
  return 0;
}
