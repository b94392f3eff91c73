// Stand-in: instantiates an operator template over both stand-in grid
// flavours (with and without a virial field) and runs execute() once in an
// uncalled function, so every operator body is compiled.
#pragma once
#include <memory>
#include "grid.h"
namespace exanb {
template <template <class> class OpT>
std::shared_ptr<::onika::scg::OperatorNode> make_grid_variant_operator() {
  auto a = std::make_shared<OpT<StubGrid<false>>>();
  auto b = std::make_shared<OpT<StubGrid<true>>>();
  a->execute();
  b->execute();
  return a;
}
}  // namespace exanb
