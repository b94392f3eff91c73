// Stand-in: EXASTAMP_CONST_QUANTITY(expr in eV, ang) -> a double.
#pragma once
#include <onika/physics/units.h>
namespace exaStamp {
namespace stub_units {
constexpr double eV = 9648.533212331;
constexpr double ang = 1.0;
}  // namespace stub_units
}  // namespace exaStamp
#define EXASTAMP_CONST_QUANTITY(E) ([] { using namespace ::exaStamp::stub_units; return double(E); }())
