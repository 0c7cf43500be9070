// ORACLE (test infrastructure only): System.Numerics semantics for the CPU restatement.
// Compiled with -ffp-contract=off; a fused multiply-add appears only where the reference calls
// FusedMultiplyAdd.  Templated on the scalar so the BSDFs can also run in double precision.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>

namespace orc {

template <class T>
struct Vec3 {
  T X, Y, Z;
  Vec3() : X(0), Y(0), Z(0) {}
  Vec3(T x, T y, T z) : X(x), Y(y), Z(z) {}
  explicit Vec3(T s) : X(s), Y(s), Z(s) {}
  T operator[](int i) const { return i == 0 ? X : (i == 1 ? Y : Z); }
  Vec3 operator+(const Vec3& b) const { return {X + b.X, Y + b.Y, Z + b.Z}; }
  Vec3 operator-(const Vec3& b) const { return {X - b.X, Y - b.Y, Z - b.Z}; }
  Vec3 operator*(const Vec3& b) const { return {X * b.X, Y * b.Y, Z * b.Z}; }
  Vec3 operator*(T s) const { return {X * s, Y * s, Z * s}; }
  Vec3 operator/(T s) const { return {X / s, Y / s, Z / s}; }
  Vec3 operator/(const Vec3& b) const { return {X / b.X, Y / b.Y, Z / b.Z}; }
  Vec3 operator-() const { return {-X, -Y, -Z}; }
  T LengthSquared() const { return Dot(*this, *this); }
  T Length() const { return std::sqrt(LengthSquared()); }
  static T Dot(const Vec3& a, const Vec3& b) { return (a.X * b.X + a.Y * b.Y) + a.Z * b.Z; }
  static Vec3 Cross(const Vec3& a, const Vec3& b) {
    return {a.Y * b.Z - a.Z * b.Y, a.Z * b.X - a.X * b.Z, a.X * b.Y - a.Y * b.X};
  }
  static Vec3 Normalize(const Vec3& a) { return a / a.Length(); }
  static Vec3 MinNative(const Vec3& a, const Vec3& b) {
    return {a.X < b.X ? a.X : b.X, a.Y < b.Y ? a.Y : b.Y, a.Z < b.Z ? a.Z : b.Z};
  }
  static Vec3 MaxNative(const Vec3& a, const Vec3& b) {
    return {a.X > b.X ? a.X : b.X, a.Y > b.Y ? a.Y : b.Y, a.Z > b.Z ? a.Z : b.Z};
  }
  static Vec3 FusedMultiplyAdd(const Vec3& a, const Vec3& b, const Vec3& c) {
    return {std::fma(a.X, b.X, c.X), std::fma(a.Y, b.Y, c.Y), std::fma(a.Z, b.Z, c.Z)};
  }
};
template <class T>
inline Vec3<T> operator*(T s, const Vec3<T>& v) { return {s * v.X, s * v.Y, s * v.Z}; }

using Vector3 = Vec3<float>;

// Math.Max / Math.Min on floats: NaN if either argument is NaN
inline float MathMax(float a, float b) {
  if (a != a || b != b) return std::numeric_limits<float>::quiet_NaN();
  return a > b ? a : b;
}
inline float MathMin(float a, float b) {
  if (a != a || b != b) return std::numeric_limits<float>::quiet_NaN();
  return a < b ? a : b;
}

// Matrix4x4, memory order M11..M44
struct Matrix4x4 {
  float m[16];
  Vector3 Translation() const { return {m[12], m[13], m[14]}; }
};
inline Vector3 Transform(const Vector3& v, const Matrix4x4& M) {
  const float* m = M.m;
  return {((v.X * m[0] + v.Y * m[4]) + v.Z * m[8]) + m[12], ((v.X * m[1] + v.Y * m[5]) + v.Z * m[9]) + m[13],
          ((v.X * m[2] + v.Y * m[6]) + v.Z * m[10]) + m[14]};
}

}  // namespace orc
