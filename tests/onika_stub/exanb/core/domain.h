// Stand-in for exaNBody's Domain and the small math types.
#pragma once
#include <onika/scg/operator.h>
namespace exanb {
struct Vec3d {
  double x = 0, y = 0, z = 0;
};
struct Mat3d {
  double m11 = 0, m12 = 0, m13 = 0, m21 = 0, m22 = 0, m23 = 0, m31 = 0, m32 = 0, m33 = 0;
};
struct AABB {
  Vec3d bmin, bmax;
};
class Domain {
 public:
  const AABB& bounds() const { return m_bounds; }
  bool periodic_boundary_x() const { return true; }
  bool periodic_boundary_y() const { return true; }
  bool periodic_boundary_z() const { return true; }
  bool xform_is_identity() const { return true; }
  const Mat3d& xform() const { return m_xform; }

 private:
  AABB m_bounds;
  Mat3d m_xform{1, 0, 0, 0, 1, 0, 0, 0, 1};
};
}  // namespace exanb
