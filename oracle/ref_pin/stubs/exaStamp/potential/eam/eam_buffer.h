// Stand-in: the math types eam_alloy.h names inside namespace exaStamp.
#pragma once
#include <onika/math/basic_types_operators.h>
namespace exaStamp {
using namespace ::onika::math;
}
