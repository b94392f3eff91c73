// Stand-in: data file paths are used as given.
#pragma once
#include <string>
namespace onika {
inline std::string data_file_path(const std::string& s) { return s; }
}  // namespace onika
