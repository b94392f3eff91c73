// Stand-in: host memory for the spline arrays.
#pragma once
#include <vector>
namespace onika {
namespace memory {
template <class T> using CudaMMVector = std::vector<T>;
}  // namespace memory
}  // namespace onika
