// Stand-in: the johnson_force parameter record (johnson.h L28-50 field names).
#pragma once
namespace exaStamp {
struct EamJohnsonParameters {
  double re, fe, rhoe, alpha, beta, A, B, kappa, lambda, Fn0, Fn1, Fn2, Fn3, F0, F1, F2, F3, Fo, eta;
};
}  // namespace exaStamp
