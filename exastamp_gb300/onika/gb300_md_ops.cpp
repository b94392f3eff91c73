// gb300_md_ops.cpp -- onika/exaNBody operator plugin that binds libgbmd.so
// (include/gbmd.h) into exaStamp's operator slots.
//
// Built as an exaStamp plugin (onika_add_plugin, as in
// src/potential/pair_potential_template/CMakeLists.txt L54-59) where onika
// and exaNBody are installed.  This repository has neither: it checks the
// file against stand-in headers of the API it uses (tests/onika_stub, a
// syntax and instantiation check) and runs the host logic, which lives in
// gb300_bridge.h, over a fake grid on the GPU (tests/onika_bridge).
//
// Force operators (drop-ins for the compute_force slot):
//   gb300_lj_force          lj_compute_force  (pair_potential_impl.hxx L104-121)
//   gb300_lj_force_symetric lj_compute_force_symetric (pair_potential_singlemat_symetric.cpp
//                           L335-346): the same forces; the half list is opt-in (half_list)
//   gb300_lj_multi_force    lj_multi_force    (pair_potential_force_op_multiparam.h L249-284)
//   gb300_eam_alloy_force   eam_alloy_force   (eam_potential_multimat.cu L88-109), with the
//                           eam_rho / eam_rho2emb / eam_force split as separate instances
//   gb300_johnson_force     johnson_force     (johnson.h, eam_potential.cu L69-193)
//   gb300_sutton_chen_force sutton_chen_force (sutton_chen.h, eam_potential.cu L69-193)
//   gb300_force             any of them, chosen by the slot `potential`
// Whole-step operators (config_numerical_schemes.msp L23-28, L44-52;
// config_move_particles.msp L116-152):
//   gb300_push_f_v_r        push_f_v_r of verlet_first_half
//   gb300_push_f_v          push_f_v of verlet_first_half / verlet_second_half
//   gb300_neighbors         check_and_update_particles (displacement trigger + rebuild)
//   gb300_sync_grid         the device state back into the grid (before thermo or dumps)
//
// All of them share one gb300::Session (device context, upload layout)
// through the slot gb300_session.  With only a force operator bound, each
// call copies the inner particles in and f = m a, ep and the virial out
// (re-uploading every field when move_particles changed the particle order,
// positions only otherwise); with the whole-step operators bound the state
// stays on the device (see gb300_bridge.h).  Each force operator keeps its
// reference operator's slot names and meaning (parameters, rcut, rcut_max,
// ghost_dist_max, chunk_neighbors, species, grid, domain,
// trigger_thermo_state, compute_virial, the eam_* pass flags), plus rcut_inc
// (the neighbour skin, global.rcut_inc) and precision (mixed or fp64).
// Slots that only steer the reference's own traversal (chunk_neighbors,
// ghost, compact_nbh_weight, enable_pair_weights, particle_locks) are
// accepted and unused.  Library errors become fatal_error(), like the
// reference operators'.
#include <onika/scg/operator.h>
#include <onika/scg/operator_factory.h>
#include <onika/scg/operator_slot.h>
#include <exanb/core/domain.h>
#include <exanb/core/grid.h>
#include <exanb/core/make_grid_variant_operator.h>
#include <exanb/particle_neighbors/chunk_neighbors.h>
#include <exaStamp/particle_species/particle_specie.h>
#include <exaStamp/potential/pair_potentials/lennard_jones/lennard_jones.h>  // LennardJonesParms + YAML
#include <exaStamp/unit_system.h>
#include <onika/physics/units.h>
#include <yaml-cpp/yaml.h>
#include "johnson.h"  // src/potential/eam_potentials/johnson (EamJohnsonParameters + its YAML decoder)
#include "sutton_chen.h"  // src/potential/eam_potentials/sutton_chen (EamSuttonChenParameters + YAML)

#include <gbmd.h>

#include "gb300_bridge.h"

#include <memory>
#include <string>
#include <vector>

namespace exaStamp {
using namespace exanb;

namespace gb300_ops {

using gb300::Field;

// The onika grid seen through gb300_bridge.h's grid-view interface: the
// inner cells in grid order, the particle fields by (cell, slot).
template <class GridT>
class GridView {
 public:
  GridView(GridT& grid, const ParticleSpecies& species) : m_grid(grid), m_species(species) {
    const IJK dims = grid.dimension();
    const ssize_t gl = grid.ghost_layers();
    GRID_FOR_BEGIN(dims - 2 * gl, _, loc) { m_inner.push_back(grid_ijk_to_index(dims, loc + gl)); }
    GRID_FOR_END
  }
  size_t inner_cells() const { return m_inner.size(); }
  size_t cell_index(size_t k) const { return m_inner[k]; }
  size_t cell_size(size_t c) const { return m_grid.cells()[c].size(); }
  double get(size_t c, Field f, size_t p) const {
    auto cells = m_grid.cells();
    switch (f) {
      case gb300::RX: return cells[c][field::rx][p];
      case gb300::RY: return cells[c][field::ry][p];
      case gb300::RZ: return cells[c][field::rz][p];
      case gb300::VX: return cells[c][field::vx][p];
      case gb300::VY: return cells[c][field::vy][p];
      case gb300::VZ: return cells[c][field::vz][p];
      case gb300::FX: return cells[c][field::fx][p];
      case gb300::FY: return cells[c][field::fy][p];
      case gb300::FZ: return cells[c][field::fz][p];
      default: return cells[c][field::ep][p];
    }
  }
  void set(size_t c, Field f, size_t p, double v) {
    auto cells = m_grid.cells();
    switch (f) {
      case gb300::RX: cells[c][field::rx][p] = v; break;
      case gb300::RY: cells[c][field::ry][p] = v; break;
      case gb300::RZ: cells[c][field::rz][p] = v; break;
      case gb300::VX: cells[c][field::vx][p] = v; break;
      case gb300::VY: cells[c][field::vy][p] = v; break;
      case gb300::VZ: cells[c][field::vz][p] = v; break;
      case gb300::FX: cells[c][field::fx][p] = v; break;
      case gb300::FY: cells[c][field::fy][p] = v; break;
      case gb300::FZ: cells[c][field::fz][p] = v; break;
      default: cells[c][field::ep][p] = v; break;
    }
  }
  uint8_t type(size_t c, size_t p) const { return m_grid.cells()[c][field::type][p]; }
  uint64_t id(size_t c, size_t p) const { return m_grid.cells()[c][field::id][p]; }
  // grid_flavor_multimat_mechanics carries the virial (grid_flavor.cpp L56-84)
  static constexpr bool kVirial = GridHasField<GridT, field::_virial>::value;
  bool has_virial() const { return kVirial; }
  void set_virial(size_t c, size_t p, const double v[9]) {
    if constexpr (kVirial) {
      Mat3d& m = m_grid.cells()[c][field::virial][p];
      m.m11 = v[0]; m.m12 = v[1]; m.m13 = v[2];
      m.m21 = v[3]; m.m22 = v[4]; m.m23 = v[5];
      m.m31 = v[6]; m.m32 = v[7]; m.m33 = v[8];
    }
  }
  double mass(int t) const { return m_species.at(t).m_mass; }

 private:
  GridT& m_grid;
  const ParticleSpecies& m_species;
  std::vector<size_t> m_inner;
};

// The domain's xform as per-axis scale factors: identity, or diagonal with
// positive entries (orthorhombic scaling, as a uniaxial deformation makes).
// A shear (off-diagonal terms) is refused.
inline void xform_scale(const Domain& domain, double scale[3]) {
  scale[0] = scale[1] = scale[2] = 1.0;
  if (domain.xform_is_identity()) return;
  const Mat3d& m = domain.xform();
  if (m.m12 != 0.0 || m.m13 != 0.0 || m.m21 != 0.0 || m.m23 != 0.0 || m.m31 != 0.0 || m.m32 != 0.0 ||
      !(m.m11 > 0.0) || !(m.m22 > 0.0) || !(m.m33 > 0.0))
    fatal_error() << "gb300: only identity or diagonal xforms (orthorhombic domains) are supported" << std::endl;
  scale[0] = m.m11;
  scale[1] = m.m22;
  scale[2] = m.m33;
}

// The shared session, created on first use with the domain and species; the
// domain's current xform is handed to it on every call.
inline gb300::Session& session_for(gb300::SessionPtr& ptr, const Domain& domain, const ParticleSpecies& species) {
  if (!ptr) ptr = std::make_shared<gb300::Session>();
  double scale[3];
  xform_scale(domain, scale);
  if (!ptr->ctx) {
    const Vec3d lo = domain.bounds().bmin, hi = domain.bounds().bmax;
    const double blo[3] = {lo.x, lo.y, lo.z}, bhi[3] = {hi.x, hi.y, hi.z};
    const int per[3] = {domain.periodic_boundary_x(), domain.periodic_boundary_y(), domain.periodic_boundary_z()};
    std::vector<double> m(species.size());
    for (size_t t = 0; t < m.size(); ++t) m[t] = species.at(t).m_mass;
    try {
      gb300::ensure_context(*ptr, parallel_execution_context()->gpu_stream(), blo, bhi, per, m, scale);
    } catch (const gb300::Error& e) {
      fatal_error() << "gb300: " << e.what() << std::endl;
    }
  }
  try {
    gb300::set_xform_scale(*ptr, scale);
  } catch (const gb300::Error& e) {
    fatal_error() << "gb300: " << e.what() << std::endl;
  }
  return *ptr;
}

// A library status as the reference operators report errors.
inline void ok(gbmd_context* c, int rc, const char* what) {
  if (rc != GBMD_OK) fatal_error() << what << " failed: " << gbmd_last_error(c) << std::endl;
}

inline void finish_setup(gb300::Session& s, double skin, const std::string& precision) {
  ok(s.ctx, gbmd_set_skin(s.ctx, skin), "gbmd_set_skin");
  ok(s.ctx, gbmd_set_precision(s.ctx, precision == "fp64" ? GBMD_PRECISION_FP64 : GBMD_PRECISION_MIXED),
               "gbmd_set_precision");
  s.potential_set = true;
}

// Runs fn(), turning library errors into fatal_error().
template <class Fn>
void guarded(const char* op, Fn&& fn) {
  try {
    fn();
  } catch (const gb300::Error& e) {
    fatal_error() << op << ": " << e.what() << std::endl;
  }
}

// One compute_force call of a force operator (per call or resident).
template <class GridT>
void compute_force_call(const char* op, gb300::Session& s, GridT& grid, const ParticleSpecies& species, bool energy,
                        bool virial, int passes) {
  GridView<GridT> view(grid, species);
  guarded(op, [&] { gb300::compute_forces(s, view, energy, virial, passes); });
}

// `parameters` of eam_alloy_force: the setfl file, as a scalar or {file: ...}
// (eam_alloy.cpp L66-84).
struct SetflRef {
  std::string file;
};

// `parameters` of lj_multi_force: [{type_a, type_b, rcut, parameters:
// {epsilon, sigma}}, ...] (pair_potential_force_op_multiparam.h L249-284).
struct LJPairEntry {
  std::string type_a, type_b;
  double rcut = 0.0;
  LennardJonesParms p;
};
struct LJPairList {
  std::vector<LJPairEntry> pairs;
};

}  // namespace gb300_ops
}  // namespace exaStamp

namespace YAML {
template <>
struct convert<exaStamp::gb300_ops::SetflRef> {
  static bool decode(const Node& node, exaStamp::gb300_ops::SetflRef& v) {
    if (node.IsScalar()) v.file = node.as<std::string>();
    else if (node.IsMap() && node["file"]) v.file = node["file"].as<std::string>();
    else return false;
    return true;
  }
};
template <>
struct convert<exaStamp::gb300_ops::LJPairList> {
  static bool decode(const Node& node, exaStamp::gb300_ops::LJPairList& v) {
    if (!node.IsSequence()) return false;
    for (auto pp : node) {
      if (!pp.IsMap() || !pp["type_a"] || !pp["type_b"] || !pp["rcut"] || !pp["parameters"]) return false;
      exaStamp::gb300_ops::LJPairEntry e;
      e.type_a = pp["type_a"].as<std::string>();
      e.type_b = pp["type_b"].as<std::string>();
      e.rcut = pp["rcut"].as<onika::physics::Quantity>().convert();
      e.p = pp["parameters"].as<exaStamp::LennardJonesParms>();
      v.pairs.push_back(e);
    }
    return true;
  }
};
}  // namespace YAML

namespace exaStamp {

using StringVector = std::vector<std::string>;
using gb300_ops::compute_force_call;
using gb300_ops::finish_setup;
using gb300_ops::session_for;

#define GB300_SESSION_SLOT \
  ADD_SLOT(gb300::SessionPtr, gb300_session, INPUT_OUTPUT, gb300::SessionPtr{}, DocString{"shared GPU context"})

// lj_compute_force (pair_potential_impl.hxx L104-121): one species pair,
// energy shifted by e(rcut) as the reference does (L373-377).  SYM: the
// lj_compute_force_symetric slots (pair_potential_singlemat_symetric.cpp
// L335-346; particle_locks accepted and unused).  The forces are the same;
// the library's full list is faster on GB300, so the Newton-3 half list
// (reaction forces through fixed-point atomics, also deterministic) is
// opt-in through half_list.
template <class GridT, bool SYM = false>
class Gb300LJForceNode : public OperatorNode {
  ADD_SLOT(LennardJonesParms, parameters, INPUT, LennardJonesParms{});
  ADD_SLOT(double, rcut, INPUT, REQUIRED);
  ADD_SLOT(double, rcut_max, INPUT_OUTPUT, 0.0);
  ADD_SLOT(exanb::GridChunkNeighbors, chunk_neighbors, INPUT, exanb::GridChunkNeighbors{}, DocString{"unused"});
  ADD_SLOT(ParticleSpecies, species, INPUT, REQUIRED);
  ADD_SLOT(std::string, type, INPUT, OPTIONAL);
  ADD_SLOT(bool, ghost, INPUT, false);
  ADD_SLOT(GridT, grid, INPUT_OUTPUT);
  ADD_SLOT(Domain, domain, INPUT, REQUIRED);
  ADD_SLOT(bool, trigger_thermo_state, INPUT, OPTIONAL);
  ADD_SLOT(bool, compute_virial, INPUT, false);
  ADD_SLOT(double, rcut_inc, INPUT, 1.0, DocString{"neighbour skin (global.rcut_inc)"});
  ADD_SLOT(std::string, precision, INPUT, std::string{"mixed"}, DocString{"mixed or fp64"});
  ADD_SLOT(bool, half_list, INPUT, false, DocString{"Newton-3 half list, reaction forces through fixed-point atomics"});
  ADD_SLOT(GridParticleLocks, particle_locks, INPUT, OPTIONAL, DocString{"unused"});
  GB300_SESSION_SLOT;

 public:
  inline void execute() override final {
    *rcut_max = std::max(*rcut, *rcut_max);
    if (grid->number_of_cells() == 0) return;
    gb300::Session& s = session_for(*gb300_session, *domain, *species);
    if (!s.potential_set) {
      gb300_ops::ok(s.ctx, gbmd_set_lj(s.ctx, parameters->epsilon, parameters->sigma, *rcut), "gbmd_set_lj");
      finish_setup(s, *rcut_inc, *precision);
      if (SYM && *half_list) {
        // the half-list kernel: mixed precision, one lane x 4 entries per load
        gb300_ops::ok(s.ctx, gbmd_set_launch_ex(s.ctx, 1, 4, 256), "gbmd_set_launch_ex");
        gb300_ops::ok(s.ctx, gbmd_set_newton3(s.ctx, 1), "gbmd_set_newton3");
      }
    }
    const bool energy = trigger_thermo_state.has_value() && *trigger_thermo_state;
    compute_force_call("gb300_lj_force", s, *grid, *species, energy, energy && *compute_virial, 0);
  }
};

// lj_multi_force (pair_potential_force_op_multiparam.h L57-118): per
// species-pair (epsilon, sigma, rcut); pairs not listed take
// common_parameters with the operator's rcut, or do not interact.
template <class GridT>
class Gb300LJMultiForceNode : public OperatorNode {
  ADD_SLOT(LennardJonesParms, common_parameters, INPUT, OPTIONAL);
  ADD_SLOT(gb300_ops::LJPairList, parameters, INPUT, REQUIRED);
  ADD_SLOT(double, rcut, INPUT, REQUIRED);
  ADD_SLOT(double, rcut_max, INPUT_OUTPUT, 0.0);
  ADD_SLOT(exanb::GridChunkNeighbors, chunk_neighbors, INPUT, exanb::GridChunkNeighbors{}, DocString{"unused"});
  ADD_SLOT(ParticleSpecies, species, INPUT, REQUIRED);
  ADD_SLOT(GridT, grid, INPUT_OUTPUT);
  ADD_SLOT(Domain, domain, INPUT, REQUIRED);
  ADD_SLOT(bool, trigger_thermo_state, INPUT, OPTIONAL);
  ADD_SLOT(bool, compute_virial, INPUT, false);
  ADD_SLOT(double, rcut_inc, INPUT, 1.0, DocString{"neighbour skin (global.rcut_inc)"});
  ADD_SLOT(std::string, precision, INPUT, std::string{"mixed"}, DocString{"mixed or fp64"});
  GB300_SESSION_SLOT;

 public:
  inline void execute() override final {
    double rmax = *rcut;
    for (const auto& e : parameters->pairs) rmax = std::max(rmax, e.rcut);
    *rcut_max = std::max(rmax, *rcut_max);
    if (grid->number_of_cells() == 0) return;
    gb300::Session& s = session_for(*gb300_session, *domain, *species);
    if (!s.potential_set) {
      const int nt = (int)species->size();
      std::vector<double> eps(nt * nt, 0.0), sig(nt * nt, 1.0), rc(nt * nt, 0.0);
      if (common_parameters.has_value())
        for (int k = 0; k < nt * nt; ++k) {
          eps[k] = common_parameters->epsilon;
          sig[k] = common_parameters->sigma;
          rc[k] = *rcut;
        }
      auto type_of = [&](const std::string& name) {
        for (int t = 0; t < nt; ++t)
          if (species->at(t).name() == name) return t;
        fatal_error() << "gb300: unknown species " << name << std::endl;
        return -1;
      };
      for (const auto& e : parameters->pairs) {
        const int a = type_of(e.type_a), b = type_of(e.type_b);
        for (int k : {a * nt + b, b * nt + a}) {
          eps[k] = e.p.epsilon;
          sig[k] = e.p.sigma;
          rc[k] = e.rcut;
        }
      }
      gb300_ops::ok(s.ctx, gbmd_set_lj_multi(s.ctx, nt, eps.data(), sig.data(), rc.data(), *rcut),
                   "gbmd_set_lj_multi");
      finish_setup(s, *rcut_inc, *precision);
    }
    const bool energy = trigger_thermo_state.has_value() && *trigger_thermo_state;
    compute_force_call("gb300_lj_multi_force", s, *grid, *species, energy, energy && *compute_virial, 0);
  }
};

// eam_alloy_force (eam_potential_multimat.cu L88-109).  The passes follow
// the eam_* flags (L101-105, L186-232): all three in one call, or split
// over operator instances as in baseline_single_specy.yaml L41-54 --
// eam_rho (density + embedding, F'(rho) kept on the device), eam_rho2emb
// alone (nothing left to do: the embedding ran with the density), eam_force
// (the force pass from the kept F'(rho), on the same positions).  The
// instances share the device context through gb300_session.  eam_ghost is
// accepted (there are no ghost cells on the device).  eam_symmetry (Newton-3
// scatter, eam_force_op_multimat.h L162-169, L305-338) runs on the full list
// by default: the same sums up to rounding, and faster on GB300.  With
// half_list it runs on the Newton-3 half list, rho_j and the reaction forces
// added through fixed-point atomics (deterministic; mixed precision).
template <class GridT>
class Gb300EamAlloyForceNode : public OperatorNode {
  ADD_SLOT(ParticleSpecies, species, INPUT, REQUIRED);
  ADD_SLOT(gb300_ops::SetflRef, parameters, INPUT, REQUIRED, DocString{"setfl file (scalar or {file: ...})"});
  ADD_SLOT(StringVector, types, INPUT, StringVector{});
  ADD_SLOT(double, rcut, INPUT, REQUIRED);
  ADD_SLOT(double, rcut_max, INPUT_OUTPUT, 0.0);
  ADD_SLOT(double, ghost_dist_max, INPUT_OUTPUT, 0.0);
  ADD_SLOT(exanb::GridChunkNeighbors, chunk_neighbors, INPUT, exanb::GridChunkNeighbors{}, DocString{"unused"});
  ADD_SLOT(GridT, grid, INPUT_OUTPUT);
  ADD_SLOT(Domain, domain, INPUT, REQUIRED);
  ADD_SLOT(bool, trigger_thermo_state, INPUT, OPTIONAL);
  ADD_SLOT(bool, compute_virial, INPUT, false);
  ADD_SLOT(bool, eam_rho, INPUT, true);
  ADD_SLOT(bool, eam_rho2emb, INPUT, true);
  ADD_SLOT(bool, eam_ghost, INPUT, true);
  ADD_SLOT(bool, eam_force, INPUT, true);
  ADD_SLOT(bool, eam_symmetry, INPUT, false, DocString{"Newton-3 scatter; on the full list unless half_list"});
  ADD_SLOT(bool, half_list, INPUT, false, DocString{"with eam_symmetry: the Newton-3 half list"});
  ADD_SLOT(double, rcut_inc, INPUT, 1.0, DocString{"neighbour skin (global.rcut_inc)"});
  ADD_SLOT(std::string, precision, INPUT, std::string{"mixed"}, DocString{"mixed or fp64"});
  GB300_SESSION_SLOT;

 public:
  inline void execute() override final {
    *rcut_max = std::max(*rcut, *rcut_max);
    *ghost_dist_max = std::max(*ghost_dist_max, 2.0 * (*rcut));
    if (grid->number_of_cells() == 0) return;
    const int passes = (*eam_rho && *eam_force) ? 0
                       : *eam_rho               ? GBMD_FORCE_PASS_DENSITY
                       : *eam_force             ? GBMD_FORCE_PASS_FORCE
                                                : -1;
    if (passes < 0) return;  // eam_rho2emb alone: the embedding already ran with the density
    gb300::Session& s = session_for(*gb300_session, *domain, *species);
    if (!s.potential_set) {
      gb300_ops::ok(s.ctx,
                   gbmd_load_setfl(s.ctx, onika::data_file_path(parameters->file).c_str(), *rcut,
                                   EXASTAMP_CONST_QUANTITY(1. * eV * ang), EXASTAMP_CONST_QUANTITY(1.0 * eV)),
                   "gbmd_load_setfl");
      finish_setup(s, *rcut_inc, *precision);
      if (*eam_symmetry && *half_list) {
        // the half-list kernels: mixed precision, one lane x 4 entries per load
        gb300_ops::ok(s.ctx, gbmd_set_launch_ex(s.ctx, 1, 4, 256), "gbmd_set_launch_ex");
        gb300_ops::ok(s.ctx, gbmd_set_newton3(s.ctx, 1), "gbmd_set_newton3");
      }
    }
    const bool energy = trigger_thermo_state.has_value() && *trigger_thermo_state;
    compute_force_call("gb300_eam_alloy_force", s, *grid, *species, energy, energy && *compute_virial, passes);
  }
};

// johnson_force (johnson.h L28-176 through the mono-material two-pass
// template, eam_potential.cu L69-193).
template <class GridT>
class Gb300JohnsonForceNode : public OperatorNode {
  ADD_SLOT(EamJohnsonParameters, parameters, INPUT, REQUIRED);
  ADD_SLOT(double, rcut, INPUT, REQUIRED);
  ADD_SLOT(double, rcut_max, INPUT_OUTPUT, 0.0);
  ADD_SLOT(double, ghost_dist_max, INPUT_OUTPUT, 0.0);
  ADD_SLOT(exanb::GridChunkNeighbors, chunk_neighbors, INPUT, exanb::GridChunkNeighbors{}, DocString{"unused"});
  ADD_SLOT(ParticleSpecies, species, INPUT, REQUIRED);
  ADD_SLOT(GridT, grid, INPUT_OUTPUT);
  ADD_SLOT(Domain, domain, INPUT, REQUIRED);
  ADD_SLOT(bool, trigger_thermo_state, INPUT, OPTIONAL);
  ADD_SLOT(bool, compute_virial, INPUT, false);
  ADD_SLOT(double, rcut_inc, INPUT, 1.0, DocString{"neighbour skin (global.rcut_inc)"});
  ADD_SLOT(std::string, precision, INPUT, std::string{"mixed"}, DocString{"mixed or fp64"});
  GB300_SESSION_SLOT;

 public:
  inline void execute() override final {
    *rcut_max = std::max(*rcut, *rcut_max);
    *ghost_dist_max = std::max(*ghost_dist_max, 2.0 * (*rcut));
    if (grid->number_of_cells() == 0) return;
    gb300::Session& s = session_for(*gb300_session, *domain, *species);
    if (!s.potential_set) {
      const EamJohnsonParameters& q = *parameters;
      const double jp[19] = {q.re, q.fe, q.rhoe, q.alpha, q.beta, q.A,   q.B,  q.kappa, q.lambda, q.Fn0,
                             q.Fn1, q.Fn2, q.Fn3, q.F0, q.F1, q.F2, q.F3, q.Fo, q.eta};
      gb300_ops::ok(s.ctx, gbmd_set_eam_johnson(s.ctx, jp, *rcut), "gbmd_set_eam_johnson");
      finish_setup(s, *rcut_inc, *precision);
    }
    const bool energy = trigger_thermo_state.has_value() && *trigger_thermo_state;
    compute_force_call("gb300_johnson_force", s, *grid, *species, energy, energy && *compute_virial, 0);
  }
};

// sutton_chen_force (sutton_chen.h L30-67 through the same template).
template <class GridT>
class Gb300SuttonChenForceNode : public OperatorNode {
  ADD_SLOT(EamSuttonChenParameters, parameters, INPUT, REQUIRED);
  ADD_SLOT(double, rcut, INPUT, REQUIRED);
  ADD_SLOT(double, rcut_max, INPUT_OUTPUT, 0.0);
  ADD_SLOT(double, ghost_dist_max, INPUT_OUTPUT, 0.0);
  ADD_SLOT(exanb::GridChunkNeighbors, chunk_neighbors, INPUT, exanb::GridChunkNeighbors{}, DocString{"unused"});
  ADD_SLOT(ParticleSpecies, species, INPUT, REQUIRED);
  ADD_SLOT(GridT, grid, INPUT_OUTPUT);
  ADD_SLOT(Domain, domain, INPUT, REQUIRED);
  ADD_SLOT(bool, trigger_thermo_state, INPUT, OPTIONAL);
  ADD_SLOT(bool, compute_virial, INPUT, false);
  ADD_SLOT(double, rcut_inc, INPUT, 1.0, DocString{"neighbour skin (global.rcut_inc)"});
  ADD_SLOT(std::string, precision, INPUT, std::string{"mixed"}, DocString{"mixed or fp64"});
  GB300_SESSION_SLOT;

 public:
  inline void execute() override final {
    *rcut_max = std::max(*rcut, *rcut_max);
    *ghost_dist_max = std::max(*ghost_dist_max, 2.0 * (*rcut));
    if (grid->number_of_cells() == 0) return;
    gb300::Session& s = session_for(*gb300_session, *domain, *species);
    if (!s.potential_set) {
      const EamSuttonChenParameters& q = *parameters;
      const double sp[5] = {q.c, q.epsilon, q.a0, q.n, q.m};
      gb300_ops::ok(s.ctx, gbmd_set_eam_sutton_chen(s.ctx, sp, *rcut), "gbmd_set_eam_sutton_chen");
      finish_setup(s, *rcut_inc, *precision);
    }
    const bool energy = trigger_thermo_state.has_value() && *trigger_thermo_state;
    compute_force_call("gb300_sutton_chen_force", s, *grid, *species, energy, energy && *compute_virial, 0);
  }
};

template <class GridT>
class Gb300ForceNode : public OperatorNode {
  ADD_SLOT(std::string, potential, INPUT, REQUIRED, DocString{"lj, eam_alloy or johnson"});
  ADD_SLOT(double, rcut, INPUT, REQUIRED);
  ADD_SLOT(double, rcut_max, INPUT_OUTPUT, 0.0);
  ADD_SLOT(double, ghost_dist_max, INPUT_OUTPUT, 0.0);
  ADD_SLOT(double, rcut_inc, INPUT, 1.0, DocString{"neighbour skin (global.rcut_inc)"});
  ADD_SLOT(double, epsilon, INPUT, 0.0);
  ADD_SLOT(double, sigma, INPUT, 0.0);
  ADD_SLOT(std::string, setfl_file, INPUT, std::string{}, DocString{"eam_alloy parameter file"});
  ADD_SLOT(EamJohnsonParameters, johnson_parameters, INPUT, OPTIONAL,
           DocString{"johnson parameters (johnson.h L28-49), as the johnson_force slot `parameters`"});
  ADD_SLOT(std::string, precision, INPUT, std::string{"mixed"}, DocString{"mixed or fp64"});
  ADD_SLOT(bool, trigger_thermo_state, INPUT, OPTIONAL);
  ADD_SLOT(bool, compute_virial, INPUT, false);
  ADD_SLOT(GridT, grid, INPUT_OUTPUT);
  ADD_SLOT(Domain, domain, INPUT, REQUIRED);
  ADD_SLOT(ParticleSpecies, species, INPUT, REQUIRED);
  GB300_SESSION_SLOT;

 public:
  inline void execute() override final {
    *rcut_max = std::max(*rcut, *rcut_max);
    if (*potential == "eam_alloy" || *potential == "johnson")
      *ghost_dist_max = std::max(*ghost_dist_max, 2.0 * (*rcut));
    if (grid->number_of_cells() == 0) return;  // pre-initialisation pass publishing rcut_max
    gb300::Session& s = session_for(*gb300_session, *domain, *species);
    if (!s.potential_set) {
      if (*potential == "lj")
        gb300_ops::ok(s.ctx, gbmd_set_lj(s.ctx, *epsilon, *sigma, *rcut), "gbmd_set_lj");
      else if (*potential == "eam_alloy")
        gb300_ops::ok(s.ctx,
                     gbmd_load_setfl(s.ctx, onika::data_file_path(*setfl_file).c_str(), *rcut,
                                     EXASTAMP_CONST_QUANTITY(1. * eV * ang), EXASTAMP_CONST_QUANTITY(1.0 * eV)),
                     "gbmd_load_setfl");
      else if (*potential == "johnson") {
        if (!johnson_parameters.has_value()) fatal_error() << "gb300: johnson needs johnson_parameters" << std::endl;
        const EamJohnsonParameters& q = *johnson_parameters;
        const double jp[19] = {q.re, q.fe, q.rhoe, q.alpha, q.beta, q.A,   q.B,  q.kappa, q.lambda, q.Fn0,
                               q.Fn1, q.Fn2, q.Fn3, q.F0, q.F1, q.F2, q.F3, q.Fo, q.eta};
        gb300_ops::ok(s.ctx, gbmd_set_eam_johnson(s.ctx, jp, *rcut), "gbmd_set_eam_johnson");
      } else
        fatal_error() << "gb300: unsupported potential " << *potential << std::endl;
      finish_setup(s, *rcut_inc, *precision);
    }
    const bool energy = trigger_thermo_state.has_value() && *trigger_thermo_state;
    compute_force_call("gb300_force", s, *grid, *species, energy, energy && *compute_virial, 0);
  }
};

// push_f_v_r / push_f_v (exaNBody push operators, scheduled by
// config_numerical_schemes.msp L23-28; formula
// push_vec3_2nd_order_xform_minimization.cpp L33-38) on the device's copy of
// the state: r += v dt' + a dt'^2 / 2 (R) or v += a dt' (V), dt' = dt dt_scale.
// With a diagonal xform the device pushes physical coordinates, and the grid
// gets them back divided by the scale: INV_XFORM for the positions,
// IDENTITY for the velocities, as the run files set xform_mode.
template <class GridT, bool R>
class Gb300PushNode : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT_OUTPUT);
  ADD_SLOT(double, dt, INPUT, REQUIRED);
  ADD_SLOT(double, dt_scale, INPUT, REQUIRED);
  ADD_SLOT(std::string, xform_mode, INPUT, std::string{"INV_XFORM"});
  ADD_SLOT(Domain, domain, INPUT, REQUIRED);
  ADD_SLOT(ParticleSpecies, species, INPUT, REQUIRED);
  GB300_SESSION_SLOT;

 public:
  inline void execute() override final {
    if (grid->number_of_cells() == 0) return;
    gb300::Session& s = session_for(*gb300_session, *domain, *species);
    gb300_ops::GridView<GridT> view(*grid, *species);
    gb300_ops::guarded(R ? "gb300_push_f_v_r" : "gb300_push_f_v", [&] {
      if (R) gb300::push_f_v_r(s, view, *dt, *dt_scale);
      else gb300::push_f_v(s, view, *dt, *dt_scale);
    });
  }
};

// check_and_update_particles (config_move_particles.msp L116-152) on the
// device's copy: trigger_move_particles (particle_displ_over against skin/2,
// L19-22) and the full update (wrap, rebin, neighbour list) when it fires.
// The outcome is published in trigger_move_particles for the graph's other
// operators (load balancing logs, counters).  list_buffer > 0 makes the
// rebuilds two-level (gbmd_set_list_buffer: the list filtered from an outer
// list of rcut + skin + list_buffer, which is rebuilt with the sort into
// cells only when an atom moved half the buffer); 0 keeps full rebuilds.
template <class GridT>
class Gb300NeighborsNode : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT_OUTPUT);
  ADD_SLOT(Domain, domain, INPUT, REQUIRED);
  ADD_SLOT(ParticleSpecies, species, INPUT, REQUIRED);
  ADD_SLOT(double, list_buffer, INPUT, 0.0, DocString{"two-level list: outer buffer beyond rcut + skin (0: off)"});
  ADD_SLOT(bool, trigger_move_particles, OUTPUT);
  GB300_SESSION_SLOT;

 public:
  inline void execute() override final {
    if (grid->number_of_cells() == 0) return;
    gb300::Session& s = session_for(*gb300_session, *domain, *species);
    gb300_ops::ok(s.ctx, gbmd_set_list_buffer(s.ctx, *list_buffer), "gbmd_set_list_buffer");
    gb300_ops::GridView<GridT> view(*grid, *species);
    bool rebuilt = false;
    gb300_ops::guarded("gb300_neighbors", [&] { rebuilt = gb300::update_neighbors(s, view); });
    *trigger_move_particles = rebuilt;
  }
};

// The device state back into the grid (whole-step runs): r, v, the
// accelerations into the f fields, and, on thermo steps, ep and the virial.
// Bound before the operators that read the grid (thermodynamic state, dumps).
template <class GridT>
class Gb300SyncGridNode : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT_OUTPUT);
  ADD_SLOT(ParticleSpecies, species, INPUT, REQUIRED);
  ADD_SLOT(bool, trigger_thermo_state, INPUT, OPTIONAL);
  ADD_SLOT(bool, compute_virial, INPUT, false);
  GB300_SESSION_SLOT;

 public:
  inline void execute() override final {
    if (!*gb300_session || grid->number_of_cells() == 0) return;
    const bool energy = trigger_thermo_state.has_value() && *trigger_thermo_state;
    gb300_ops::GridView<GridT> view(*grid, *species);
    gb300_ops::guarded("gb300_sync_grid",
                       [&] { gb300::sync_grid(**gb300_session, view, energy, energy && *compute_virial); });
  }
};

template <class GridT>
using Gb300ForceNodeTmpl = Gb300ForceNode<GridT>;
template <class GridT>
using Gb300LJForceTmpl = Gb300LJForceNode<GridT>;
template <class GridT>
using Gb300LJForceSymTmpl = Gb300LJForceNode<GridT, true>;
template <class GridT>
using Gb300LJMultiForceTmpl = Gb300LJMultiForceNode<GridT>;
template <class GridT>
using Gb300EamAlloyForceTmpl = Gb300EamAlloyForceNode<GridT>;
template <class GridT>
using Gb300JohnsonForceTmpl = Gb300JohnsonForceNode<GridT>;
template <class GridT>
using Gb300SuttonChenForceTmpl = Gb300SuttonChenForceNode<GridT>;
template <class GridT>
using Gb300PushFVRTmpl = Gb300PushNode<GridT, true>;
template <class GridT>
using Gb300PushFVTmpl = Gb300PushNode<GridT, false>;
template <class GridT>
using Gb300NeighborsTmpl = Gb300NeighborsNode<GridT>;
template <class GridT>
using Gb300SyncGridTmpl = Gb300SyncGridNode<GridT>;

ONIKA_AUTORUN_INIT(gb300_md_ops) {
  OperatorNodeFactory::instance()->register_factory("gb300_force", make_grid_variant_operator<Gb300ForceNodeTmpl>);
  OperatorNodeFactory::instance()->register_factory("gb300_lj_force", make_grid_variant_operator<Gb300LJForceTmpl>);
  OperatorNodeFactory::instance()->register_factory("gb300_lj_force_symetric",
                                                    make_grid_variant_operator<Gb300LJForceSymTmpl>);
  OperatorNodeFactory::instance()->register_factory("gb300_lj_multi_force",
                                                    make_grid_variant_operator<Gb300LJMultiForceTmpl>);
  OperatorNodeFactory::instance()->register_factory("gb300_eam_alloy_force",
                                                    make_grid_variant_operator<Gb300EamAlloyForceTmpl>);
  OperatorNodeFactory::instance()->register_factory("gb300_johnson_force",
                                                    make_grid_variant_operator<Gb300JohnsonForceTmpl>);
  OperatorNodeFactory::instance()->register_factory("gb300_sutton_chen_force",
                                                    make_grid_variant_operator<Gb300SuttonChenForceTmpl>);
  OperatorNodeFactory::instance()->register_factory("gb300_push_f_v_r", make_grid_variant_operator<Gb300PushFVRTmpl>);
  OperatorNodeFactory::instance()->register_factory("gb300_push_f_v", make_grid_variant_operator<Gb300PushFVTmpl>);
  OperatorNodeFactory::instance()->register_factory("gb300_neighbors", make_grid_variant_operator<Gb300NeighborsTmpl>);
  OperatorNodeFactory::instance()->register_factory("gb300_sync_grid", make_grid_variant_operator<Gb300SyncGridTmpl>);
}

}  // namespace exaStamp
