#include "host_math.hpp"

#include <cmath>
#include <limits>

namespace bnh {

bool m4_invert(const M4& in, M4* out) {
  // Laplace expansion: the six 2x2 minors of the lower two rows give the cofactors of the
  // first row (and the determinant); the minors of rows 1-2 and 1-3... give the rest.
  const float* q = in.m;
  const float a = q[0], b = q[1], c = q[2], d = q[3];
  const float e = q[4], f = q[5], g = q[6], h = q[7];
  const float i = q[8], j = q[9], k = q[10], l = q[11];
  const float m = q[12], n = q[13], o = q[14], p = q[15];

  const float m34_a = k * p - l * o, m34_b = j * p - l * n, m34_c = j * o - k * n;
  const float m34_d = i * p - l * m, m34_e = i * o - k * m, m34_f = i * n - j * m;

  const float c11 = (f * m34_a - g * m34_b) + h * m34_c;
  const float c12 = -((e * m34_a - g * m34_d) + h * m34_e);
  const float c13 = (e * m34_b - f * m34_d) + h * m34_f;
  const float c14 = -((e * m34_c - f * m34_e) + g * m34_f);
  const float det = ((a * c11 + b * c12) + c * c13) + d * c14;
  if (std::fabs(det) < std::numeric_limits<float>::denorm_min()) {
    const float nan = std::numeric_limits<float>::quiet_NaN();
    for (int z = 0; z < 16; ++z) out->m[z] = nan;
    return false;
  }
  const float inv = 1.f / det;
  float* r = out->m;
  r[0] = c11 * inv;
  r[4] = c12 * inv;
  r[8] = c13 * inv;
  r[12] = c14 * inv;
  r[1] = -((b * m34_a - c * m34_b) + d * m34_c) * inv;
  r[5] = ((a * m34_a - c * m34_d) + d * m34_e) * inv;
  r[9] = -((a * m34_b - b * m34_d) + d * m34_f) * inv;
  r[13] = ((a * m34_c - b * m34_e) + c * m34_f) * inv;

  const float m24_a = g * p - h * o, m24_b = f * p - h * n, m24_c = f * o - g * n;
  const float m24_d = e * p - h * m, m24_e = e * o - g * m, m24_f = e * n - f * m;
  r[2] = ((b * m24_a - c * m24_b) + d * m24_c) * inv;
  r[6] = -((a * m24_a - c * m24_d) + d * m24_e) * inv;
  r[10] = ((a * m24_b - b * m24_d) + d * m24_f) * inv;
  r[14] = -((a * m24_c - b * m24_e) + c * m24_f) * inv;

  const float m23_a = g * l - h * k, m23_b = f * l - h * j, m23_c = f * k - g * j;
  const float m23_d = e * l - h * i, m23_e = e * k - g * i, m23_f = e * j - f * i;
  r[3] = -((b * m23_a - c * m23_b) + d * m23_c) * inv;
  r[7] = ((a * m23_a - c * m23_d) + d * m23_e) * inv;
  r[11] = -((a * m23_b - b * m23_d) + d * m23_f) * inv;
  r[15] = ((a * m23_c - b * m23_e) + c * m23_f) * inv;
  return true;
}

void det_sincos(double x, double* s, double* c) {
  // x = k * (pi/2) + r with |r| <= pi/4; pi/2 is split in two parts so that k * hi is exact
  // for the small k the generators need.
  const double half_pi_hi = 1.5707963267341256;      // 33 significant bits of pi/2
  const double half_pi_lo = 6.077100506506192e-11;   // pi/2 - half_pi_hi
  const double kd = std::floor(x / 1.5707963267948966 + 0.5);
  const double r = (x - kd * half_pi_hi) - kd * half_pi_lo;
  const double r2 = r * r;
  // Taylor series to r^19 / r^18: truncation below 1e-17 for |r| <= pi/4
  double sn = 0.0, cs = 0.0;
  {
    double term = r;
    sn = term;
    for (int n = 1; n <= 9; ++n) {
      term = -term * r2 / static_cast<double>((2 * n) * (2 * n + 1));
      sn = sn + term;
    }
    term = 1.0;
    cs = term;
    for (int n = 1; n <= 9; ++n) {
      term = -term * r2 / static_cast<double>((2 * n - 1) * (2 * n));
      cs = cs + term;
    }
  }
  long long k = static_cast<long long>(kd);
  int q = static_cast<int>(((k % 4) + 4) % 4);
  switch (q) {
    case 0: *s = sn; *c = cs; break;
    case 1: *s = cs; *c = -sn; break;
    case 2: *s = -sn; *c = -cs; break;
    default: *s = -cs; *c = sn; break;
  }
}

}  // namespace bnh
