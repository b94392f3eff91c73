// Stand-in for the part of yaml-cpp the plugin's decoders use.
#pragma once
#include <string>
#include <vector>
namespace YAML {
class Node {
 public:
  bool IsScalar() const;
  bool IsMap() const;
  bool IsSequence() const;
  Node operator[](const char*) const;
  explicit operator bool() const;
  template <class T>
  T as() const;
  std::vector<Node>::const_iterator begin() const;
  std::vector<Node>::const_iterator end() const;
};
template <class T>
struct convert;
}  // namespace YAML
