// Stand-in for the read-only shallow-copy trait eam_alloy.h specialises.
#pragma once
namespace onika {
namespace cuda {
template <class T> struct ReadOnlyShallowCopyType { using type = T; };
}  // namespace cuda
}  // namespace onika
