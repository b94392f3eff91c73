// Stand-in for onika's Vec3d / Mat3d with the operations the per-atom force
// loop and eam_alloy_mm_force use: Vec3d *= s, Mat3d += Mat3d, Mat3d * s,
// tensor(u, v) (the outer product u v^T), is_zero.
#pragma once
namespace onika {
namespace math {
struct Vec3d {
  double x = 0.0, y = 0.0, z = 0.0;
  Vec3d& operator*=(double s) {
    x *= s;
    y *= s;
    z *= s;
    return *this;
  }
};
struct Mat3d {
  double m11 = 0, m12 = 0, m13 = 0, m21 = 0, m22 = 0, m23 = 0, m31 = 0, m32 = 0, m33 = 0;
  Mat3d& operator+=(const Mat3d& b) {
    m11 += b.m11; m12 += b.m12; m13 += b.m13;
    m21 += b.m21; m22 += b.m22; m23 += b.m23;
    m31 += b.m31; m32 += b.m32; m33 += b.m33;
    return *this;
  }
};
inline Mat3d operator*(const Mat3d& a, double s) {
  return Mat3d{a.m11 * s, a.m12 * s, a.m13 * s, a.m21 * s, a.m22 * s, a.m23 * s, a.m31 * s, a.m32 * s, a.m33 * s};
}
inline Mat3d tensor(const Vec3d& u, const Vec3d& v) {
  return Mat3d{u.x * v.x, u.x * v.y, u.x * v.z, u.y * v.x, u.y * v.y, u.y * v.z, u.z * v.x, u.z * v.y, u.z * v.z};
}
inline bool is_zero(const Mat3d& a) {
  return a.m11 == 0 && a.m12 == 0 && a.m13 == 0 && a.m21 == 0 && a.m22 == 0 && a.m23 == 0 && a.m31 == 0 &&
         a.m32 == 0 && a.m33 == 0;
}
}  // namespace math
}  // namespace onika
namespace exanb {
using namespace ::onika::math;
}
