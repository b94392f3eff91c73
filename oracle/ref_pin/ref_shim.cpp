// ref_shim.cpp -- C entry points around the reference's own per-pair code,
// compiled from the exaStamp sources in place (see build_ref.py) with the
// stand-ins of stubs/ for onika and yaml-cpp.  Test infrastructure only: the
// oracle's restatement is compared with these functions bit for bit
// (tests/test_ref_pin.py); nothing of the product links this library.
//
// Compiled reference code:
//   lennard_jones.h L41-50          lj_compute_energy
//   force_op_impl2.hxx L22-78       the per-atom loop of lj_compute_force over a
//                                   filled pair buffer (included below into a
//                                   function body that provides its names)
//   eam_alloy.cpp L29-278           setfl reader and 7-coefficient splines
//   eam_alloy.h L198-313            eam_alloy_rho_noderiv, eam_alloy_mm_force,
//                                   eam_alloy_fEmbed
#include <cstdint>
#include <cstring>
#include <memory>

#include <exaStamp/potential/pair_potentials/lennard_jones/lennard_jones.h>

#include "eam_alloy.h"

using exaStamp::EamAlloyParameters;
using exaStamp::EamAlloyParametersRO;
using onika::math::Mat3d;
using onika::math::Vec3d;

namespace {

// The pair buffer the force loop reads (ComputePairBuffer2's arrays) and a
// weight source of 1 (no pair weighting).
struct PairBuffer {
  const double *drx, *dry, *drz, *d2;
  struct NoWeights {
    double get(size_t) const { return 1.0; }
  } nbh_data;
};

std::unique_ptr<EamAlloyParameters> g_eam;
std::unique_ptr<EamAlloyParametersRO> g_eam_ro;

}  // namespace

extern "C" {

void ref_lj_compute_energy(double epsilon, double sigma, double r, double* e, double* de) {
  const exaStamp::LennardJonesParms p{epsilon, sigma};
  const exaStamp::PairPotentialMinimalParameters pp{};
  exaStamp::lj_compute_energy(p, pp, r, *e, *de);
}

// One atom of lj_compute_force: out = {ep, fx, fy, fz, vir[9] row-major}.
void ref_lj_force_atom(double epsilon, double sigma, double ecut, int n_, const double* drx, const double* dry,
                       const double* drz, const double* d2, double* out) {
  using namespace onika::math;
  const exaStamp::LennardJonesParms p{epsilon, sigma};
  const exaStamp::PairPotentialMinimalParameters pair_params{};
  const PairBuffer tab{drx, dry, drz, d2, {}};
  const size_t n = (size_t)n_;
  double ep = 0.0, ax = 0.0, ay = 0.0, az = 0.0;
  Mat3d virial;
#define USTAMP_POTENTIAL_COMPUTE(p_, pp_, r_, e_, de_) exaStamp::lj_compute_energy(p_, pp_, r_, e_, de_)
#include "force_op_impl2.hxx"
#undef USTAMP_POTENTIAL_COMPUTE
  out[0] = ep;
  out[1] = ax;
  out[2] = ay;
  out[3] = az;
  const double v[9] = {virial.m11, virial.m12, virial.m13, virial.m21, virial.m22,
                       virial.m23, virial.m31, virial.m32, virial.m33};
  std::memcpy(out + 4, v, sizeof(v));
}

// eam_alloy setfl file -> spline tables (eam_alloy.cpp's decoder), with the
// type tables of initialize_types_table for the file's elements.  Returns
// the element count (0 on failure); nr, nrho receive the table sizes.
int ref_eam_load(const char* path, int* nr, int* nrho) {
  g_eam.reset(new EamAlloyParameters());
  YAML::Node node{std::string(path)};
  if (!YAML::convert<EamAlloyParameters>::decode(node, *g_eam)) return 0;
  g_eam->initialize_types_table(g_eam->nelements, nullptr);
  g_eam_ro.reset(new EamAlloyParametersRO(*g_eam));
  *nr = g_eam->nr;
  *nrho = g_eam->nrho;
  return g_eam->nelements;
}

// Flattened spline coefficients (8 doubles per knot) of table `which`
// (0 F(rho), 1 rho(r), 2 z2r) into out; returns the number of knots.
int64_t ref_eam_spline(int which, double* out) {
  const auto& v = which == 0 ? g_eam->frho_spline_data : (which == 1 ? g_eam->rhor_spline_data : g_eam->z2r_spline_data);
  if (out)
    for (size_t k = 0; k < v.size(); ++k) std::memcpy(out + 8 * k, v[k].coeffs, 8 * sizeof(double));
  return (int64_t)v.size();
}

void ref_eam_conversions(double* conv_z2r, double* conv_frho) {
  *conv_z2r = EamAlloyParametersRO::conversion_z2r;
  *conv_frho = EamAlloyParametersRO::conversion_frho;
}

double ref_eam_rho(double r, int itype, int jtype) { return exaStamp::eam_alloy_rho_noderiv(*g_eam_ro, r, itype, jtype); }

// eam_alloy_mm_force: dr is scaled in place by fpair; phi receives phi(r).
void ref_eam_mm_force(double r, double fpi, double fpj, int itype, int jtype, double* dr, double* phi) {
  Vec3d v{dr[0], dr[1], dr[2]};
  exaStamp::eam_alloy_mm_force(*g_eam_ro, v, *phi, r, fpi, fpj, itype, jtype);
  dr[0] = v.x;
  dr[1] = v.y;
  dr[2] = v.z;
}

void ref_eam_fembed(double rho, int itype, double* phi, double* fp) {
  exaStamp::eam_alloy_fEmbed(*g_eam_ro, rho, *phi, *fp, itype);
}

}  // extern "C"
