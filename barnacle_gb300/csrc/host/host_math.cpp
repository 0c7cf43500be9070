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

// ---- System.Numerics restatements for keyframe interpolation (Base/Scene.fs:13-20)

namespace {
float length3(V3 v) { return std::sqrt((v.x * v.x + v.y * v.y) + v.z * v.z); }
V3 normalize3(V3 v) {
  const float l = length3(v);
  return {v.x / l, v.y / l, v.z / l};
}
V3 cross3(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
}  // namespace

// Matrix4x4.GetDeterminant: expansion along the first row over the 2x2 minors of rows 3-4
float m4_determinant(const M4& M) {
  const float* q = M.m;
  const float a = q[0], b = q[1], c = q[2], d = q[3];
  const float e = q[4], f = q[5], g = q[6], h = q[7];
  const float i = q[8], j = q[9], k = q[10], l = q[11];
  const float m = q[12], n = q[13], o = q[14], p = q[15];
  const float kp_lo = k * p - l * o, jp_ln = j * p - l * n, jo_kn = j * o - k * n;
  const float ip_lm = i * p - l * m, io_km = i * o - k * m, in_jm = i * n - j * m;
  return a * (f * kp_lo - g * jp_ln + h * jo_kn) - b * (e * kp_lo - g * ip_lm + h * io_km) +
         c * (e * jp_ln - f * ip_lm + h * in_jm) - d * (e * jo_kn - f * io_km + g * in_jm);
}

// Quaternion.CreateFromRotationMatrix: the trace branch, else the largest diagonal element's
static void quat_from_rotation(const M4& M, float q[4]) {
  const float* m = M.m;
  const float m11 = m[0], m12 = m[1], m13 = m[2], m21 = m[4], m22 = m[5], m23 = m[6], m31 = m[8], m32 = m[9],
              m33 = m[10];
  const float trace = m11 + m22 + m33;
  if (trace > 0.f) {
    float s = std::sqrt(trace + 1.f);
    q[3] = s * 0.5f;
    s = 0.5f / s;
    q[0] = (m23 - m32) * s;
    q[1] = (m31 - m13) * s;
    q[2] = (m12 - m21) * s;
  } else if (m11 >= m22 && m11 >= m33) {
    const float s = std::sqrt(1.f + m11 - m22 - m33), inv = 0.5f / s;
    q[0] = 0.5f * s;
    q[1] = (m12 + m21) * inv;
    q[2] = (m13 + m31) * inv;
    q[3] = (m23 - m32) * inv;
  } else if (m22 > m33) {
    const float s = std::sqrt(1.f + m22 - m11 - m33), inv = 0.5f / s;
    q[0] = (m21 + m12) * inv;
    q[1] = 0.5f * s;
    q[2] = (m32 + m23) * inv;
    q[3] = (m31 - m13) * inv;
  } else {
    const float s = std::sqrt(1.f + m33 - m11 - m22), inv = 0.5f / s;
    q[0] = (m31 + m13) * inv;
    q[1] = (m32 + m23) * inv;
    q[2] = 0.5f * s;
    q[3] = (m12 - m21) * inv;
  }
}

// Matrix4x4.Decompose: row lengths are the scales; the rows are ranked by length, a row shorter
// than 1e-4 is replaced (canonical axis, or a cross product), all are normalised, a negative
// determinant flips the longest; |det - 1|^2 > 1e-4 marks a matrix that is not SRT
bool m4_decompose(const M4& M, V3* scale, float rot[4], V3* translation) {
  constexpr float kEps = 0.0001f;
  const float* m = M.m;
  *translation = {m[12], m[13], m[14]};
  V3 basis[3] = {{m[0], m[1], m[2]}, {m[4], m[5], m[6]}, {m[8], m[9], m[10]}};
  const V3 canonical[3] = {{1.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, {0.f, 0.f, 1.f}};
  float sc[3] = {length3(basis[0]), length3(basis[1]), length3(basis[2])};
  int a, b, c;
  const float x = sc[0], y = sc[1], z = sc[2];
  if (x < y) {
    if (y < z) { a = 2; b = 1; c = 0; }
    else { a = 1; if (x < z) { b = 2; c = 0; } else { b = 0; c = 2; } }
  } else {
    if (x < z) { a = 2; b = 0; c = 1; }
    else { a = 0; if (y < z) { b = 2; c = 1; } else { b = 1; c = 2; } }
  }
  if (sc[a] < kEps) basis[a] = canonical[a];
  basis[a] = normalize3(basis[a]);
  if (sc[b] < kEps) {
    const float ax = std::fabs(basis[a].x), ay = std::fabs(basis[a].y), az = std::fabs(basis[a].z);
    int cc;
    if (ax < ay) cc = (ay < az) ? 0 : (ax < az ? 0 : 2);
    else cc = (ax < az) ? 1 : (ay < az ? 1 : 2);
    basis[b] = cross3(basis[a], canonical[cc]);
  }
  basis[b] = normalize3(basis[b]);
  if (sc[c] < kEps) basis[c] = cross3(basis[a], basis[b]);
  basis[c] = normalize3(basis[c]);
  M4 tmp = m4_identity();
  for (int r = 0; r < 3; ++r) {
    tmp.m[4 * r] = basis[r].x;
    tmp.m[4 * r + 1] = basis[r].y;
    tmp.m[4 * r + 2] = basis[r].z;
  }
  float det = m4_determinant(tmp);
  if (det < 0.f) {
    sc[a] = -sc[a];
    basis[a] = {-basis[a].x, -basis[a].y, -basis[a].z};
    tmp.m[4 * a] = basis[a].x;
    tmp.m[4 * a + 1] = basis[a].y;
    tmp.m[4 * a + 2] = basis[a].z;
    det = -det;
  }
  det -= 1.f;
  det *= det;
  *scale = {sc[0], sc[1], sc[2]};
  if (kEps < det) {
    rot[0] = rot[1] = rot[2] = 0.f;
    rot[3] = 1.f;
    return false;
  }
  quat_from_rotation(tmp, rot);
  return true;
}

// Matrix4x4.CreateFromQuaternion
M4 m4_from_quaternion(const float q[4]) {
  const float xx = q[0] * q[0], yy = q[1] * q[1], zz = q[2] * q[2];
  const float xy = q[0] * q[1], wz = q[2] * q[3], xz = q[2] * q[0], wy = q[1] * q[3], yz = q[1] * q[2],
              wx = q[0] * q[3];
  M4 r = m4_identity();
  r.m[0] = 1.f - 2.f * (yy + zz);
  r.m[1] = 2.f * (xy + wz);
  r.m[2] = 2.f * (xz - wy);
  r.m[4] = 2.f * (xy - wz);
  r.m[5] = 1.f - 2.f * (zz + xx);
  r.m[6] = 2.f * (yz + wx);
  r.m[8] = 2.f * (xz + wy);
  r.m[9] = 2.f * (yz - wx);
  r.m[10] = 1.f - 2.f * (yy + xx);
  return r;
}

// Quaternion.Slerp: the shorter arc (sign flip), linear weights within 1e-6 of parallel
void quat_slerp(const float a[4], const float b[4], float t, float out[4]) {
  constexpr float kEps = 1e-6f;
  float cos_omega = ((a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]) + a[3] * b[3];
  bool flip = false;
  if (cos_omega < 0.f) {
    flip = true;
    cos_omega = -cos_omega;
  }
  float s1, s2;
  if (cos_omega > 1.f - kEps) {
    s1 = 1.f - t;
    s2 = flip ? -t : t;
  } else {
    const float omega = std::acos(cos_omega);
    const float inv_sin = 1.f / std::sin(omega);
    s1 = std::sin((1.f - t) * omega) * inv_sin;
    s2 = flip ? -std::sin(t * omega) * inv_sin : std::sin(t * omega) * inv_sin;
  }
  for (int k = 0; k < 4; ++k) out[k] = s1 * a[k] + s2 * b[k];
}

M4 keyframe_interpolate(float ta, const M4& A, float tb, const M4& B, float t) {
  const float ratio = (t - ta) / (tb - ta);
  V3 s1, s2, t1, t2;
  float r1[4], r2[4], r[4];
  m4_decompose(A, &s1, r1, &t1);
  m4_decompose(B, &s2, r2, &t2);
  // Vector3.Lerp(a, b, w) = a * (1 - w) + b * w
  auto lerp = [](V3 a, V3 b, float w) {
    return V3{a.x * (1.f - w) + b.x * w, a.y * (1.f - w) + b.y * w, a.z * (1.f - w) + b.z * w};
  };
  const V3 trans = lerp(t1, t2, ratio);
  quat_slerp(r1, r2, ratio, r);
  const V3 scale = lerp(s1, s2, ratio);
  // Transform.Compose(scale, rotation, translation): translation matrix from `scale`, scale
  // matrix from `translation`, as the reference composes them
  return m4_mul(m4_mul(m4_translation(scale.x, scale.y, scale.z), m4_from_quaternion(r)),
                m4_scale(trans.x, trans.y, trans.z));
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
