// Stand-in for exanb::lout: a stream without a buffer (writes are dropped).
#pragma once
#include <ostream>
namespace exanb {
inline std::ostream lout(nullptr);
}  // namespace exanb
