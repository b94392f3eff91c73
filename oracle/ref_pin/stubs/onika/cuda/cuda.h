// Stand-in: host-only build, so the host/device decorations are empty.
#pragma once
#include <cassert>
#define ONIKA_HOST_DEVICE_FUNC
#define ONIKA_ALWAYS_INLINE inline __attribute__((always_inline))
