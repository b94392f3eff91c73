// Stand-in for onika's operator factory and its autorun registration hook.
#pragma once
#include <functional>
#include <memory>
#include <string>
#include "operator.h"

namespace onika {
namespace scg {
class OperatorNodeFactory {
 public:
  static OperatorNodeFactory* instance();
  void register_factory(const std::string& name, std::shared_ptr<OperatorNode> (*make)());
};
}  // namespace scg
}  // namespace onika

#define ONIKA_AUTORUN_INIT(name) static void onika_autorun_##name()
