// Stand-in for yaml-cpp: a node that is either empty or one scalar string
// (the setfl file path eam_alloy's decoder reads), and the convert<> hook.
#pragma once
#include <cstdint>
#include <limits>
#include <string>
#include <vector>

namespace YAML {
class Node {
 public:
  Node() = default;
  explicit Node(const std::string& s) : scalar_(s), has_(true) {}
  bool IsScalar() const { return has_; }
  bool IsMap() const { return false; }
  Node operator[](const char*) const { return Node(); }
  explicit operator bool() const { return has_; }
  template <class T> T as() const;

 private:
  std::string scalar_;
  bool has_ = false;
};
template <> inline std::string Node::as<std::string>() const { return scalar_; }
template <class T> struct convert;
}  // namespace YAML
