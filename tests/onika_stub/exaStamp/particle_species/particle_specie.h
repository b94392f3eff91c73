// Stand-in for exaStamp's species table (m_mass, name()).
#pragma once
#include <string>
#include <vector>
namespace exaStamp {
struct ParticleSpecie {
  double m_mass = 1.0;
  std::string m_name;
  const std::string& name() const { return m_name; }
};
using ParticleSpecies = std::vector<ParticleSpecie>;
}  // namespace exaStamp
