// Stand-in: lennard_jones.h only passes PairPotentialMinimalParameters through.
#pragma once
#include <onika/math/basic_types_operators.h>
namespace exanb {}
namespace exaStamp {
using namespace exanb;
struct PairPotentialMinimalParameters {};
}  // namespace exaStamp
