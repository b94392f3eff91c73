// Stand-in: the sutton_chen_force parameter record (sutton_chen.h L30-37 field names).
#pragma once
namespace exaStamp {
struct EamSuttonChenParameters {
  double c, epsilon, a0, n, m;
};
}  // namespace exaStamp
