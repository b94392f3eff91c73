// Stand-in: nothing of onika's physical constants is used by the compiled code.
#pragma once
#include "units.h"
