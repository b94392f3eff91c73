// Stand-in for onika's unit system: quantities are stored directly in the
// reference's internal units (angstrom, dalton, picosecond), so converting
// to that system is the identity.  eV uses the CODATA 2018 values
// (1.602176634e-19 J, 1 Da = 1.66053906660e-27 kg), as the build's systems.py.
#pragma once

namespace onika {
namespace physics {
struct UnitDef {
  int id;
};
constexpr UnitDef angstrom{0}, atomic_mass_unit{1}, picosecond{2}, elementary_charge{3}, kelvin{4}, particle{5},
    candela{6}, radian{7};
struct UnitSystem {
  UnitDef units[8];
};
struct Quantity {
  double value = 0.0;
  constexpr double convert(const UnitSystem&) const { return value; }
  constexpr double convert() const { return value; }
};
constexpr Quantity operator*(double a, Quantity q) { return Quantity{a * q.value}; }
constexpr Quantity operator*(Quantity a, Quantity b) { return Quantity{a.value * b.value}; }
namespace stub_units {
constexpr Quantity eV{1.602176634e-19 / 1.66053906660e-23};  // Da A^2 / ps^2
constexpr Quantity ang{1.0};
}  // namespace stub_units
}  // namespace physics
}  // namespace onika

#define ONIKA_CONST_QUANTITY(E) ([]() constexpr { using namespace ::onika::physics::stub_units; return (E); }())
#define ONIKA_QUANTITY(E) ONIKA_CONST_QUANTITY(E)
