// gb300_md_ops.cpp -- onika/exaNBody operator plugin that binds libgbmd.so
// (include/gbmd.h) into exaStamp's operator slots.
//
// Built as an exaStamp plugin (onika_add_plugin, as in
// src/potential/pair_potential_template/CMakeLists.txt L54-59) when onika and
// exaNBody are available; it is not compiled in this repository, which has
// neither.  Operator:
//
//   gb300_force   drop-in for lj_compute_force / eam_alloy_force in the
//                 compute_force slot (slot `potential`: lj or eam_alloy)
//
// It keeps the reference slots (pair_potential_impl.hxx
// L104-121, eam_potential_multimat.cu L88-109): rcut, rcut_max, parameters,
// ghost_dist_max, grid, domain, species, trigger_thermo_state,
// compute_virial.  Each execute() copies the inner-cell particles
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
#include <exaStamp/particle_species/particle_specie.h>
#include <exaStamp/unit_system.h>
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

}  // namespace gb300

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
      gbmd_context* c = nullptr;
      if (gbmd_create(&c, 0, parallel_execution_context()->gpu_stream()) != GBMD_OK)
        fatal_error() << "gb300: no GPU context" << std::endl;
      m_ctx.reset(c);
      const Vec3d lo = domain->bounds().bmin, hi = domain->bounds().bmax;
      const double blo[3] = {lo.x, lo.y, lo.z}, bhi[3] = {hi.x, hi.y, hi.z};
      const int per[3] = {domain->periodic_boundary_x(), domain->periodic_boundary_y(), domain->periodic_boundary_z()};
      gb300::check(c, gbmd_set_box(c, blo, bhi, per), "gbmd_set_box");
      std::vector<double> m(species->size());
      for (size_t t = 0; t < m.size(); ++t) m[t] = species->at(t).m_mass;
      gb300::check(c, gbmd_set_species(c, (int)m.size(), m.data()), "gbmd_set_species");
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
      gb300::check(c, gbmd_set_skin(c, *rcut_inc), "gbmd_set_skin");
      gb300::check(c, gbmd_set_precision(c, *precision == "fp64" ? GBMD_PRECISION_FP64 : GBMD_PRECISION_MIXED),
                   "gbmd_set_precision");
    }
    gbmd_context* c = m_ctx.get();
    gb300::Staging& s = m_stage;
    gb300::gather(*grid, s);
    if (s.n != m_uploaded) {
      gb300::check(c, gbmd_upload_atoms(c, (int64_t)s.n, s.rx.data(), s.ry.data(), s.rz.data(), s.vx.data(),
                                        s.vy.data(), s.vz.data(), s.type.data(), s.id.data()),
                   "gbmd_upload_atoms");
      m_uploaded = s.n;
    } else {
      gb300::check(c, gbmd_upload_positions(c, s.rx.data(), s.ry.data(), s.rz.data(), nullptr, nullptr, nullptr),
                   "gbmd_upload_positions");
    }
    const bool energy = trigger_thermo_state.has_value() && *trigger_thermo_state;
    const bool virial = energy && *compute_virial;
    gb300::check(c, gbmd_compute_forces(c, (energy ? GBMD_FORCE_ENERGY : 0) | (virial ? GBMD_FORCE_VIRIAL : 0)),
                 "gbmd_compute_forces");
    gb300::check(c, gbmd_download(c, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, s.ax.data(), s.ay.data(),
                                  s.az.data(), energy ? s.ep.data() : nullptr, virial ? s.vir.data() : nullptr),
                 "gbmd_download");
    auto cells = grid->cells();
    for (size_t k = 0; k < s.n; ++k) {
      const size_t cc = s.cell_of[k], p = s.slot_of[k];
      const double m = species->at(s.type[k]).m_mass;
      cells[cc][field::fx][p] = s.ax[k] * m;  // force_to_accel runs next in the graph
      cells[cc][field::fy][p] = s.ay[k] * m;
      cells[cc][field::fz][p] = s.az[k] * m;
      if (energy) cells[cc][field::ep][p] = s.ep[k];
    }
  }
};

template <class GridT>
using Gb300ForceNodeTmpl = Gb300ForceNode<GridT>;

ONIKA_AUTORUN_INIT(gb300_md_ops) {
  OperatorNodeFactory::instance()->register_factory("gb300_force", make_grid_variant_operator<Gb300ForceNodeTmpl>);
}

}  // namespace exaStamp
