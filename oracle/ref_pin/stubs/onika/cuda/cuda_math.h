// Stand-in for onika::cuda::min / max (plain comparisons).
#pragma once
namespace onika {
namespace cuda {
template <class T> constexpr T min(T a, T b) { return a < b ? a : b; }
template <class T> constexpr T max(T a, T b) { return a > b ? a : b; }
}  // namespace cuda
}  // namespace onika
