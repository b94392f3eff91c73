// Stand-in: the Lennard-Jones parameter pair the plugin reads.
#pragma once
#include <yaml-cpp/yaml.h>
namespace exaStamp {
struct LennardJonesParms {
  double epsilon = 0.0;
  double sigma = 0.0;
};
}  // namespace exaStamp
