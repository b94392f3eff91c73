// gb300_md_ops.cpp -- onika/exaNBody operator plugin that binds libgbmd.so
// (include/gbmd.h) into exaStamp's operator slots.
//
// Built as an exaStamp plugin (onika_add_plugin, as in
// src/potential/pair_potential_template/CMakeLists.txt L54-59) when onika and
// exaNBody are available; it is not compiled in this repository, which has
// neither.  Operators (drop-ins for the compute_force slot):
//
//   gb300_lj_force         lj_compute_force  (pair_potential_impl.hxx L104-121)
//   gb300_lj_force_symetric lj_compute_force_symetric (pair_potential_singlemat_symetric.cpp L335-346):
//                          the same with the Newton-3 half list (gbmd_set_newton3)
//   gb300_lj_multi_force   lj_multi_force    (pair_potential_force_op_multiparam.h L249-284)
//   gb300_eam_alloy_force  eam_alloy_force   (eam_potential_multimat.cu L88-109)
//   gb300_johnson_force    johnson_force     (johnson.h, eam_potential.cu L69-193)
//   gb300_force            any of them, chosen by the slot `potential`
//
// Each keeps its reference operator's slot names and meaning (parameters,
// rcut, rcut_max, ghost_dist_max, chunk_neighbors, species, grid, domain,
// trigger_thermo_state, compute_virial, the eam_* pass flags), plus rcut_inc
// (the neighbour skin, global.rcut_inc) and precision (mixed or fp64).
// Slots that only steer the reference's own traversal (chunk_neighbors,
// ghost, compact_nbh_weight, enable_pair_weights) are accepted and unused:
// the library keeps its own list, rebuilt on the skin/2 displacement test.  Each execute() copies the inner-cell particles
// (rx,ry,rz,vx,vy,vz,type,id) into the GPU context, runs zero_force_energy +
// compute_force + force_to_accel on the device, and writes forces f = m*a,
// ep and virial back into the cells, so the graph's own force_to_accel and
// push operators keep working unchanged.  Errors become fatal_error(), like
// the reference operators.
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

#include <gbmd.h>

#include <memory>
#include <string>
#include <vector>

namespace exaStamp {
using namespace exanb;

namespace gb300 {

struct ContextDeleter {
  void operator()(gbmd_context* c) const { gbmd_destroy(c); }
};
using ContextPtr = std::unique_ptr<gbmd_context, ContextDeleter>;

inline void check(gbmd_context* c, int rc, const char* what) {
  if (rc != GBMD_OK) fatal_error() << what << " failed: " << gbmd_last_error(c) << std::endl;
}

// Host staging of the inner cells' particles in a fixed (cell, slot) order.
struct Staging {
  std::vector<double> rx, ry, rz, vx, vy, vz, ax, ay, az, ep, vir;
  std::vector<uint8_t> type;
  std::vector<uint64_t> id;
  std::vector<size_t> cell_of, slot_of;
  size_t n = 0;
};

template <class GridT>
void gather(const GridT& grid, Staging& s) {
  auto cells = grid.cells();
  const IJK dims = grid.dimension();
  const ssize_t gl = grid.ghost_layers();
  s = Staging{};
  GRID_FOR_BEGIN(dims - 2 * gl, _, loc) {
    const size_t c = grid_ijk_to_index(dims, loc + gl);
    const size_t np = cells[c].size();
    for (size_t p = 0; p < np; ++p) {
      s.rx.push_back(cells[c][field::rx][p]);
      s.ry.push_back(cells[c][field::ry][p]);
      s.rz.push_back(cells[c][field::rz][p]);
      s.vx.push_back(cells[c][field::vx][p]);
      s.vy.push_back(cells[c][field::vy][p]);
      s.vz.push_back(cells[c][field::vz][p]);
      s.type.push_back(cells[c][field::type][p]);
      s.id.push_back(cells[c][field::id][p]);
      s.cell_of.push_back(c);
      s.slot_of.push_back(p);
    }
  }
  GRID_FOR_END
  s.n = s.rx.size();
  s.ax.resize(s.n);
  s.ay.resize(s.n);
  s.az.resize(s.n);
  s.ep.resize(s.n);
  s.vir.resize(9 * s.n);
}

inline gbmd_context* make_context(const Domain& domain, const ParticleSpecies& species) {
  gbmd_context* c = nullptr;
  if (gbmd_create(&c, 0, parallel_execution_context()->gpu_stream()) != GBMD_OK)
    fatal_error() << "gb300: no GPU context" << std::endl;
  const Vec3d lo = domain.bounds().bmin, hi = domain.bounds().bmax;
  const double blo[3] = {lo.x, lo.y, lo.z}, bhi[3] = {hi.x, hi.y, hi.z};
  const int per[3] = {domain.periodic_boundary_x(), domain.periodic_boundary_y(), domain.periodic_boundary_z()};
  check(c, gbmd_set_box(c, blo, bhi, per), "gbmd_set_box");
  std::vector<double> m(species.size());
  for (size_t t = 0; t < m.size(); ++t) m[t] = species.at(t).m_mass;
  check(c, gbmd_set_species(c, (int)m.size(), m.data()), "gbmd_set_species");
  return c;
}

inline void finish_setup(gbmd_context* c, double skin, const std::string& precision) {
  check(c, gbmd_set_skin(c, skin), "gbmd_set_skin");
  check(c, gbmd_set_precision(c, precision == "fp64" ? GBMD_PRECISION_FP64 : GBMD_PRECISION_MIXED),
        "gbmd_set_precision");
}

// One compute_force call: the inner cells' particles into the context
// (all of them when the count changed, else positions only: the library's
// skin/2 displacement test decides a rebuild), zero_force_energy +
// compute_force + force_to_accel on the device, then f = m a and ep back into
// the cells (the graph's force_to_accel runs next).
template <class GridT>
void compute_and_store(gbmd_context* c, GridT& grid, const ParticleSpecies& species, Staging& s, size_t& uploaded,
                       bool energy, bool virial) {
  gather(grid, s);
  if (s.n != uploaded) {
    check(c, gbmd_upload_atoms(c, (int64_t)s.n, s.rx.data(), s.ry.data(), s.rz.data(), s.vx.data(), s.vy.data(),
                               s.vz.data(), s.type.data(), s.id.data()),
          "gbmd_upload_atoms");
    uploaded = s.n;
  } else {
    check(c, gbmd_upload_positions(c, s.rx.data(), s.ry.data(), s.rz.data(), nullptr, nullptr, nullptr),
          "gbmd_upload_positions");
  }
  check(c, gbmd_compute_forces(c, (energy ? GBMD_FORCE_ENERGY : 0) | (virial ? GBMD_FORCE_VIRIAL : 0)),
        "gbmd_compute_forces");
  check(c, gbmd_download(c, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, s.ax.data(), s.ay.data(),
                         s.az.data(), energy ? s.ep.data() : nullptr, virial ? s.vir.data() : nullptr),
        "gbmd_download");
  auto cells = grid.cells();
  for (size_t k = 0; k < s.n; ++k) {
    const size_t cc = s.cell_of[k], p = s.slot_of[k];
    const double m = species.at(s.type[k]).m_mass;
    cells[cc][field::fx][p] = s.ax[k] * m;
    cells[cc][field::fy][p] = s.ay[k] * m;
    cells[cc][field::fz][p] = s.az[k] * m;
    if (energy) cells[cc][field::ep][p] = s.ep[k];
  }
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

}  // namespace gb300
}  // namespace exaStamp

namespace YAML {
template <>
struct convert<exaStamp::gb300::SetflRef> {
  static bool decode(const Node& node, exaStamp::gb300::SetflRef& v) {
    if (node.IsScalar()) v.file = node.as<std::string>();
    else if (node.IsMap() && node["file"]) v.file = node["file"].as<std::string>();
    else return false;
    return true;
  }
};
template <>
struct convert<exaStamp::gb300::LJPairList> {
  static bool decode(const Node& node, exaStamp::gb300::LJPairList& v) {
    if (!node.IsSequence()) return false;
    for (auto pp : node) {
      if (!pp.IsMap() || !pp["type_a"] || !pp["type_b"] || !pp["rcut"] || !pp["parameters"]) return false;
      exaStamp::gb300::LJPairEntry e;
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

// lj_compute_force (pair_potential_impl.hxx L104-121): one species pair,
// energy shifted by e(rcut) as the reference does (L373-377).  SYM: the
// lj_compute_force_symetric slots (pair_potential_singlemat_symetric.cpp
// L335-346; particle_locks accepted and unused: the library scatters the
// reaction forces with atomics) on the Newton-3 half list.
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
  ADD_SLOT(GridParticleLocks, particle_locks, INPUT, OPTIONAL, DocString{"unused (atomic scatter)"});
  gb300::ContextPtr m_ctx;
  gb300::Staging m_stage;
  size_t m_uploaded = 0;

 public:
  inline void execute() override final {
    *rcut_max = std::max(*rcut, *rcut_max);
    if (grid->number_of_cells() == 0) return;
    if (!m_ctx) {
      gbmd_context* c = gb300::make_context(*domain, *species);
      m_ctx.reset(c);
      gb300::check(c, gbmd_set_lj(c, parameters->epsilon, parameters->sigma, *rcut), "gbmd_set_lj");
      gb300::finish_setup(c, *rcut_inc, *precision);
      if (SYM) {
        // the half-list kernel: mixed precision, one lane x 4 entries per load
        gb300::check(c, gbmd_set_launch_ex(c, 1, 4, 256), "gbmd_set_launch_ex");
        gb300::check(c, gbmd_set_newton3(c, 1), "gbmd_set_newton3");
      }
    }
    const bool energy = trigger_thermo_state.has_value() && *trigger_thermo_state;
    gb300::compute_and_store(m_ctx.get(), *grid, *species, m_stage, m_uploaded, energy, energy && *compute_virial);
  }
};

// lj_multi_force (pair_potential_force_op_multiparam.h L57-118): per
// species-pair (epsilon, sigma, rcut); pairs not listed take
// common_parameters with the operator's rcut, or do not interact.
template <class GridT>
class Gb300LJMultiForceNode : public OperatorNode {
  ADD_SLOT(LennardJonesParms, common_parameters, INPUT, OPTIONAL);
  ADD_SLOT(gb300::LJPairList, parameters, INPUT, REQUIRED);
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
  gb300::ContextPtr m_ctx;
  gb300::Staging m_stage;
  size_t m_uploaded = 0;

 public:
  inline void execute() override final {
    double rmax = *rcut;
    for (const auto& e : parameters->pairs) rmax = std::max(rmax, e.rcut);
    *rcut_max = std::max(rmax, *rcut_max);
    if (grid->number_of_cells() == 0) return;
    if (!m_ctx) {
      gbmd_context* c = gb300::make_context(*domain, *species);
      m_ctx.reset(c);
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
      gb300::check(c, gbmd_set_lj_multi(c, nt, eps.data(), sig.data(), rc.data(), *rcut), "gbmd_set_lj_multi");
      gb300::finish_setup(c, *rcut_inc, *precision);
    }
    const bool energy = trigger_thermo_state.has_value() && *trigger_thermo_state;
    gb300::compute_and_store(m_ctx.get(), *grid, *species, m_stage, m_uploaded, energy, energy && *compute_virial);
  }
};

// eam_alloy_force (eam_potential_multimat.cu L88-109): the three passes in
// one call; the split-pass and Newton-3 forms are not offered.
template <class GridT>
class Gb300EamAlloyForceNode : public OperatorNode {
  ADD_SLOT(ParticleSpecies, species, INPUT, REQUIRED);
  ADD_SLOT(gb300::SetflRef, parameters, INPUT, REQUIRED, DocString{"setfl file (scalar or {file: ...})"});
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
  ADD_SLOT(bool, eam_symmetry, INPUT, false);
  ADD_SLOT(double, rcut_inc, INPUT, 1.0, DocString{"neighbour skin (global.rcut_inc)"});
  ADD_SLOT(std::string, precision, INPUT, std::string{"mixed"}, DocString{"mixed or fp64"});
  gb300::ContextPtr m_ctx;
  gb300::Staging m_stage;
  size_t m_uploaded = 0;

 public:
  inline void execute() override final {
    *rcut_max = std::max(*rcut, *rcut_max);
    *ghost_dist_max = std::max(*ghost_dist_max, 2.0 * (*rcut));
    if (grid->number_of_cells() == 0) return;
    if (!(*eam_rho && *eam_rho2emb && *eam_force) || *eam_symmetry)
      fatal_error() << "gb300_eam_alloy_force: only the fused three-pass full-list form is offered" << std::endl;
    if (!m_ctx) {
      gbmd_context* c = gb300::make_context(*domain, *species);
      m_ctx.reset(c);
      gb300::check(c,
                   gbmd_load_setfl(c, onika::data_file_path(parameters->file).c_str(), *rcut,
                                   EXASTAMP_CONST_QUANTITY(1. * eV * ang), EXASTAMP_CONST_QUANTITY(1.0 * eV)),
                   "gbmd_load_setfl");
      gb300::finish_setup(c, *rcut_inc, *precision);
    }
    const bool energy = trigger_thermo_state.has_value() && *trigger_thermo_state;
    gb300::compute_and_store(m_ctx.get(), *grid, *species, m_stage, m_uploaded, energy, energy && *compute_virial);
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
  gb300::ContextPtr m_ctx;
  gb300::Staging m_stage;
  size_t m_uploaded = 0;

 public:
  inline void execute() override final {
    *rcut_max = std::max(*rcut, *rcut_max);
    *ghost_dist_max = std::max(*ghost_dist_max, 2.0 * (*rcut));
    if (grid->number_of_cells() == 0) return;
    if (!m_ctx) {
      gbmd_context* c = gb300::make_context(*domain, *species);
      m_ctx.reset(c);
      const EamJohnsonParameters& q = *parameters;
      const double jp[19] = {q.re, q.fe, q.rhoe, q.alpha, q.beta, q.A,   q.B,  q.kappa, q.lambda, q.Fn0,
                             q.Fn1, q.Fn2, q.Fn3, q.F0, q.F1, q.F2, q.F3, q.Fo, q.eta};
      gb300::check(c, gbmd_set_eam_johnson(c, jp, *rcut), "gbmd_set_eam_johnson");
      gb300::finish_setup(c, *rcut_inc, *precision);
    }
    const bool energy = trigger_thermo_state.has_value() && *trigger_thermo_state;
    gb300::compute_and_store(m_ctx.get(), *grid, *species, m_stage, m_uploaded, energy, energy && *compute_virial);
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

  gb300::ContextPtr m_ctx;
  gb300::Staging m_stage;
  size_t m_uploaded = 0;

 public:
  inline void execute() override final {
    *rcut_max = std::max(*rcut, *rcut_max);
    if (*potential == "eam_alloy" || *potential == "johnson")
      *ghost_dist_max = std::max(*ghost_dist_max, 2.0 * (*rcut));
    if (grid->number_of_cells() == 0) return;  // pre-initialisation pass publishing rcut_max
    if (!m_ctx) {
      gbmd_context* c = gb300::make_context(*domain, *species);
      m_ctx.reset(c);
      if (*potential == "lj")
        gb300::check(c, gbmd_set_lj(c, *epsilon, *sigma, *rcut), "gbmd_set_lj");
      else if (*potential == "eam_alloy")
        gb300::check(c,
                     gbmd_load_setfl(c, onika::data_file_path(*setfl_file).c_str(), *rcut,
                                     EXASTAMP_CONST_QUANTITY(1. * eV * ang), EXASTAMP_CONST_QUANTITY(1.0 * eV)),
                     "gbmd_load_setfl");
      else if (*potential == "johnson") {
        if (!johnson_parameters.has_value()) fatal_error() << "gb300: johnson needs johnson_parameters" << std::endl;
        const EamJohnsonParameters& q = *johnson_parameters;
        const double jp[19] = {q.re, q.fe, q.rhoe, q.alpha, q.beta, q.A,   q.B,  q.kappa, q.lambda, q.Fn0,
                               q.Fn1, q.Fn2, q.Fn3, q.F0, q.F1, q.F2, q.F3, q.Fo, q.eta};
        gb300::check(c, gbmd_set_eam_johnson(c, jp, *rcut), "gbmd_set_eam_johnson");
      } else
        fatal_error() << "gb300: unsupported potential " << *potential << std::endl;
      gb300::finish_setup(c, *rcut_inc, *precision);
    }
    const bool energy = trigger_thermo_state.has_value() && *trigger_thermo_state;
    gb300::compute_and_store(m_ctx.get(), *grid, *species, m_stage, m_uploaded, energy, energy && *compute_virial);
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
}

}  // namespace exaStamp
