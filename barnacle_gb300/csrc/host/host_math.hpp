// Host-side vector/matrix arithmetic with System.Numerics semantics.
//
// The scene preparation (BVH build, instance bounds, camera constants) must produce the same
// float bits as the reference's .NET code, so every operation is written out in a fixed order
// and this code is compiled with -ffp-contract=off (no fused multiply-add unless spelled out).
//  - Vector3.Transform(v, M)  = ((v.x*M11 + v.y*M21) + v.z*M31) + M41  (row-vector convention)
//  - MinNative / MaxNative   = x86 minps / maxps: (a < b ? a : b), (a > b ? a : b)
//  - Matrix4x4 product       = row i of A times B, summed left to right
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace bnh {

struct V3 {
  float x, y, z;
};
static inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
static inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
static inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
static inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static inline float length(V3 a) { return std::sqrt(dot(a, a)); }
static inline V3 normalize(V3 a) { return a / length(a); }
static inline float min_native(float a, float b) { return a < b ? a : b; }
static inline float max_native(float a, float b) { return a > b ? a : b; }
static inline V3 min_native(V3 a, V3 b) { return {min_native(a.x, b.x), min_native(a.y, b.y), min_native(a.z, b.z)}; }
static inline V3 max_native(V3 a, V3 b) { return {max_native(a.x, b.x), max_native(a.y, b.y), max_native(a.z, b.z)}; }
static inline float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// Matrix4x4 in memory order M11..M44 (m[4*(r-1) + (c-1)]).
struct M4 {
  float m[16];
};
static inline M4 m4_identity() {
  M4 r{};
  r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.f;
  return r;
}
static inline M4 m4_zero() { return M4{}; }
static inline M4 m4_mul(const M4& a, const M4& b) {
  M4 r;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      float s = a.m[4 * i + 0] * b.m[0 + j];
      s = s + a.m[4 * i + 1] * b.m[4 + j];
      s = s + a.m[4 * i + 2] * b.m[8 + j];
      s = s + a.m[4 * i + 3] * b.m[12 + j];
      r.m[4 * i + j] = s;
    }
  return r;
}
static inline M4 m4_scale(float x, float y, float z) {
  M4 r = m4_identity();
  r.m[0] = x; r.m[5] = y; r.m[10] = z;
  return r;
}
static inline M4 m4_translation(float x, float y, float z) {
  M4 r = m4_identity();
  r.m[12] = x; r.m[13] = y; r.m[14] = z;
  return r;
}
// Matrix4x4.CreateRotationX/Y/Z from a cosine/sine pair (radians in the reference).
static inline M4 m4_rot_x(float c, float s) {
  M4 r = m4_identity();
  r.m[5] = c; r.m[6] = s; r.m[9] = -s; r.m[10] = c;
  return r;
}
static inline M4 m4_rot_y(float c, float s) {
  M4 r = m4_identity();
  r.m[0] = c; r.m[2] = -s; r.m[8] = s; r.m[10] = c;
  return r;
}
static inline M4 m4_rot_z(float c, float s) {
  M4 r = m4_identity();
  r.m[0] = c; r.m[1] = s; r.m[4] = -s; r.m[5] = c;
  return r;
}
static inline V3 transform_point(V3 v, const M4& M) {
  const float* m = M.m;
  return {((v.x * m[0] + v.y * m[4]) + v.z * m[8]) + m[12],
          ((v.x * m[1] + v.y * m[5]) + v.z * m[9]) + m[13],
          ((v.x * m[2] + v.y * m[6]) + v.z * m[10]) + m[14]};
}
static inline V3 translation(const M4& M) { return {M.m[12], M.m[13], M.m[14]}; }

// Matrix4x4.Invert: cofactor expansion over 2x2 sub-determinants, then multiplication by
// 1/det.  Returns false (and a NaN matrix, as System.Numerics does) when |det| < eps.
bool m4_invert(const M4& in, M4* out);

// KeyFrame.Interpolate (Base/Scene.fs:13-20) for a render time between two keyframes: ratio =
// (t - ta) / (tb - ta); Matrix4x4.Decompose of both matrices into (scale, rotation, translation);
// Vector3.Lerp of scales and translations, Quaternion.Slerp of rotations; then
// Transform.Compose(scale, rotation, translation) (Util/Transform.fs:6-9), which builds
// CreateTranslation(scale) * CreateFromQuaternion(rotation) * CreateScale(translation) — the
// reference swaps scale and translation there, and that is kept.  The System.Numerics routines
// (.NET 9 BCL, not vendored) are restated from their published source.
M4 keyframe_interpolate(float ta, const M4& a, float tb, const M4& b, float t);
// Matrix4x4.Decompose: false for a matrix that is not scale-rotation-translation
bool m4_decompose(const M4& m, V3* scale, float rotation[4], V3* translation);
M4 m4_from_quaternion(const float q[4]);
void quat_slerp(const float a[4], const float b[4], float t, float out[4]);
float m4_determinant(const M4& m);

// Deterministic sine/cosine in double precision (range reduction + Taylor series).  The
// procedural scene generators use it so that the generated geometry has the same bits on
// every host, whatever its libm.
void det_sincos(double x, double* s, double* c);

}  // namespace bnh
