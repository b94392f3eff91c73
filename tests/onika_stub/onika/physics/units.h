// Stand-in for onika's physical quantities: a value already in internal units.
#pragma once
namespace onika {
namespace physics {
struct Quantity {
  double value = 0.0;
  double convert() const { return value; }
};
}  // namespace physics
}  // namespace onika
