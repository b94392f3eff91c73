// gb300_bridge.h -- the host logic between an exaNBody cell grid and
// libgbmd (include/gbmd.h), written without onika so that the same code
// runs in the onika plugin (gb300_md_ops.cpp) and in its tests over a fake
// grid.
//
// A grid view G adapts the grid.  It provides:
//   size_t inner_cells() const;            inner (non-ghost) cells, in grid order
//   size_t cell_index(size_t k) const;     grid index of the k-th inner cell
//   size_t cell_size(size_t c) const;      particles in cell c
//   double get(size_t c, Field f, size_t p) const;
//   void   set(size_t c, Field f, size_t p, double v);
//   uint8_t  type(size_t c, size_t p) const;
//   uint64_t id(size_t c, size_t p) const;
//   bool has_virial() const;               the grid carries a per-particle virial field
//   void set_virial(size_t c, size_t p, const double v[9]);
//   double mass(int type) const;
//
// Two ways to run a step (both keep the reference operators' slot semantics):
//
// * Per call (the compute_force slot only; the graph's own push, neighbour
//   and force_to_accel operators stay): every call gathers the inner
//   particles into the session's staging arrays, uploads them -- all fields
//   when the particle count or the particle order changed (move_particles
//   re-bins and reorders particles at every full update, also at constant
//   count), positions only otherwise (the library keeps its neighbour list
//   unless some atom moved more than skin/2) -- computes
//   zero_force_energy + compute_force + force_to_accel on the device and
//   writes f = m a, ep and, when asked and present, the virial back into the
//   cells (force_to_accel then runs on the host as usual).
// * Resident (the run file binds the push operators of verlet_first_half /
//   verlet_second_half, check_and_update_particles and compute_force to the
//   gb300 operators): the first of them uploads the grid's state (r, v, and
//   the accelerations the f fields hold after force_to_accel), after which
//   the pushes, the displacement-triggered rebuild and the forces all run on
//   the device's copy; gb300_sync_grid writes r, v, a (into the f fields),
//   ep and the virial back where a step needs the grid (thermo, dumps).
#pragma once
#include <gbmd.h>

#include <cstdint>
#include <cmath>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace gb300 {

// Library errors; the plugin turns them into fatal_error().
struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

inline void check(gbmd_context* c, int rc, const char* what) {
  if (rc != GBMD_OK) throw Error(std::string(what) + " failed: " + (c ? gbmd_last_error(c) : "no context"));
}

enum Field { RX = 0, RY, RZ, VX, VY, VZ, FX, FY, FZ, EP };

// One simulation's device context plus the layout of its last upload.  The
// operators of one run file share it through a slot.
struct Session {
  gbmd_context* ctx = nullptr;
  bool potential_set = false;
  // layout of the last upload: particle k sits at (cell[k], slot[k]) with id ids[k]
  std::vector<uint64_t> ids;
  std::vector<uint32_t> cell, slot;
  size_t n = 0;
  bool uploaded = false;
  bool resident = false;      // the device holds the current state (whole-step operators)
  bool grid_stale = false;    // the device state changed since the last write-back
  bool density_fresh = false; // a split EAM density pass ran on the uploaded positions
  int64_t full_uploads = 0, position_uploads = 0;  // counters (tests and logs)
  // diagonal xform of the domain: physical coordinates = scale x grid
  // coordinates (the device works in physical ones); next_scale is the
  // domain's current one, applied before the next device work
  double scale[3] = {1.0, 1.0, 1.0}, next_scale[3] = {1.0, 1.0, 1.0};
  double glo[3] = {0.0, 0.0, 0.0}, ghi[3] = {0.0, 0.0, 0.0};  // domain bounds, grid coordinates
  int periodic[3] = {1, 1, 1};
  // staging, reused from call to call
  std::vector<double> r[3], v[3], a[3], ep, vir;
  std::vector<uint8_t> type;
  std::vector<uint64_t> id_now;
  std::vector<uint32_t> cell_now, slot_now;

  Session() = default;
  Session(const Session&) = delete;
  Session& operator=(const Session&) = delete;
  ~Session() {
    if (ctx) gbmd_destroy(ctx);
  }
};
using SessionPtr = std::shared_ptr<Session>;

inline void check_scale(const double scale[3]) {
  for (int d = 0; d < 3; ++d)
    if (!(scale[d] > 0.0) || !std::isfinite(scale[d])) throw Error("xform scale factors must be positive and finite");
}

// The physical box of the session's bounds and current scale.
inline void set_physical_box(Session& s) {
  double lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = s.glo[d] * s.scale[d];
    hi[d] = s.ghi[d] * s.scale[d];
  }
  check(s.ctx, gbmd_set_box(s.ctx, lo, hi, s.periodic), "gbmd_set_box");
}

// The device context of the session, created on first use: device 0 on the
// given stream (may be null), box [lo, hi) in grid coordinates (fully
// periodic), species masses, and the domain's diagonal xform (scale; null:
// identity).
inline void ensure_context(Session& s, void* stream, const double lo[3], const double hi[3], const int periodic[3],
                           const std::vector<double>& masses, const double* scale = nullptr) {
  if (s.ctx) return;
  if (scale) check_scale(scale);
  gbmd_context* c = nullptr;
  const int rc = gbmd_create(&c, 0, stream);
  if (rc != GBMD_OK) throw Error("gbmd_create failed (no GPU?)");
  s.ctx = c;
  for (int d = 0; d < 3; ++d) {
    s.glo[d] = lo[d];
    s.ghi[d] = hi[d];
    s.periodic[d] = periodic[d];
    s.scale[d] = s.next_scale[d] = scale ? scale[d] : 1.0;
  }
  set_physical_box(s);
  check(c, gbmd_set_species(c, (int)masses.size(), masses.data()), "gbmd_set_species");
}

// The domain's current diagonal xform (a deformation run changes it between
// operator calls); applied before the session's next device work.
inline void set_xform_scale(Session& s, const double scale[3]) {
  check_scale(scale);
  for (int d = 0; d < 3; ++d) s.next_scale[d] = scale[d];
}

// The inner particles' layout and positions (velocities too with `with_v`)
// into the staging arrays, by index (no per-particle reallocation).
template <class G>
void gather(Session& s, const G& g, bool with_v) {
  size_t n = 0;
  const size_t nc = g.inner_cells();
  for (size_t k = 0; k < nc; ++k) n += g.cell_size(g.cell_index(k));
  for (int d = 0; d < 3; ++d) {
    s.r[d].resize(n);
    if (with_v) s.v[d].resize(n);
  }
  s.type.resize(n);
  s.id_now.resize(n);
  s.cell_now.resize(n);
  s.slot_now.resize(n);
  size_t q = 0;
  for (size_t k = 0; k < nc; ++k) {
    const size_t c = g.cell_index(k);
    const size_t np = g.cell_size(c);
    for (size_t p = 0; p < np; ++p, ++q) {
      s.r[0][q] = g.get(c, RX, p) * s.scale[0];
      s.r[1][q] = g.get(c, RY, p) * s.scale[1];
      s.r[2][q] = g.get(c, RZ, p) * s.scale[2];
      if (with_v) {
        s.v[0][q] = g.get(c, VX, p);
        s.v[1][q] = g.get(c, VY, p);
        s.v[2][q] = g.get(c, VZ, p);
      }
      s.type[q] = g.type(c, p);
      s.id_now[q] = g.id(c, p);
      s.cell_now[q] = (uint32_t)c;
      s.slot_now[q] = (uint32_t)p;
    }
  }
}

// True when the gathered particles are the uploaded ones in the same order
// (same count, same ids at every index).
inline bool same_layout(const Session& s) {
  return s.uploaded && s.id_now.size() == s.n &&
         (s.n == 0 || std::memcmp(s.id_now.data(), s.ids.data(), s.n * sizeof(uint64_t)) == 0);
}

inline void record_layout(Session& s) {
  s.n = s.id_now.size();
  s.ids = s.id_now;
  s.cell = s.cell_now;
  s.slot = s.slot_now;
  s.uploaded = true;
}

// Per-call upload: every field when the layout changed, positions otherwise.
template <class G>
void upload_for_forces(Session& s, const G& g) {
  gather(s, g, true);
  if (!same_layout(s)) {
    check(s.ctx, gbmd_upload_atoms(s.ctx, (int64_t)s.id_now.size(), s.r[0].data(), s.r[1].data(), s.r[2].data(),
                                   s.v[0].data(), s.v[1].data(), s.v[2].data(), s.type.data(), s.id_now.data()),
          "gbmd_upload_atoms");
    record_layout(s);
    ++s.full_uploads;
  } else {
    check(s.ctx, gbmd_upload_positions(s.ctx, s.r[0].data(), s.r[1].data(), s.r[2].data(), nullptr, nullptr, nullptr),
          "gbmd_upload_positions");
    ++s.position_uploads;
  }
}

// Accelerations, ep and virial of the device into the cells of the last
// upload's layout: f = m a (as_force) or a itself (the grid's f fields hold
// accelerations after force_to_accel).
template <class G>
void write_forces(Session& s, G& g, bool energy, bool virial, bool as_force) {
  const size_t n = s.n;
  for (int d = 0; d < 3; ++d) s.a[d].resize(n);
  if (energy) s.ep.resize(n);
  const bool vir = virial && g.has_virial();
  if (vir) s.vir.resize(9 * n);
  check(s.ctx, gbmd_download(s.ctx, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, s.a[0].data(), s.a[1].data(),
                             s.a[2].data(), energy ? s.ep.data() : nullptr, vir ? s.vir.data() : nullptr),
        "gbmd_download");
  // non-finite or out-of-range forces, list overflow: the reference aborts
  check(s.ctx, gbmd_check_errors(s.ctx), "gbmd_check_errors");
  for (size_t k = 0; k < n; ++k) {
    const size_t c = s.cell[k], p = s.slot[k];
    const double m = as_force ? g.mass(s.type[k]) : 1.0;
    g.set(c, FX, p, s.a[0][k] * m);
    g.set(c, FY, p, s.a[1][k] * m);
    g.set(c, FZ, p, s.a[2][k] * m);
    if (energy) g.set(c, EP, p, s.ep[k]);
    if (vir) g.set_virial(c, p, &s.vir[9 * k]);
  }
}

template <class G>
void sync_grid(Session& s, G& g, bool energy, bool virial);

// A changed xform (set_xform_scale) before new device work: the device's
// state, newer than the grid's, goes back into the grid with the old scale
// (r, v and the accelerations; energies and virials are recomputed by the
// next force call), the physical box follows the new scale, and the next
// call uploads every field again.  Grid coordinates do not change: the
// atoms move with the deformation.
template <class G>
void apply_xform(Session& s, G& g) {
  if (s.scale[0] == s.next_scale[0] && s.scale[1] == s.next_scale[1] && s.scale[2] == s.next_scale[2]) return;
  if (s.resident && s.grid_stale) sync_grid(s, g, false, false);
  s.resident = false;
  s.uploaded = false;
  s.density_fresh = false;
  for (int d = 0; d < 3; ++d) s.scale[d] = s.next_scale[d];
  set_physical_box(s);
}

// Flags of a force call: energy (trigger_thermo_state), virial
// (compute_virial) and the split EAM pass bits.
inline int force_flags(bool energy, bool virial, int passes) {
  return (energy ? GBMD_FORCE_ENERGY : 0) | (virial ? GBMD_FORCE_VIRIAL : 0) | passes;
}

// One compute_force call.  passes: 0 (all), GBMD_FORCE_PASS_DENSITY or
// GBMD_FORCE_PASS_FORCE (eam_rho / eam_force as separate operator calls on
// the same positions: the force pass reuses the density pass's upload).
template <class G>
void compute_forces(Session& s, G& g, bool energy, bool virial, int passes) {
  apply_xform(s, g);
  if (s.resident) {
    check(s.ctx, gbmd_compute_forces(s.ctx, force_flags(energy, virial, passes)), "gbmd_compute_forces");
    s.grid_stale = true;
    return;
  }
  const bool reuse = passes == GBMD_FORCE_PASS_FORCE && s.density_fresh;
  if (!reuse) upload_for_forces(s, g);
  check(s.ctx, gbmd_compute_forces(s.ctx, force_flags(energy, virial, passes)), "gbmd_compute_forces");
  s.density_fresh = passes == GBMD_FORCE_PASS_DENSITY;
  if (passes != GBMD_FORCE_PASS_DENSITY) write_forces(s, g, energy, virial, true);
}

// Resident mode from now on: the grid's full state goes to the device once.
// The f fields are taken as accelerations (the state after force_to_accel).
template <class G>
void make_resident(Session& s, const G& g) {
  if (s.resident) return;
  gather(s, g, true);
  const size_t n = s.id_now.size();
  for (int d = 0; d < 3; ++d) s.a[d].resize(n);
  size_t q = 0;
  const size_t nc = g.inner_cells();
  for (size_t k = 0; k < nc; ++k) {
    const size_t c = g.cell_index(k);
    for (size_t p = 0; p < g.cell_size(c); ++p, ++q) {
      s.a[0][q] = g.get(c, FX, p);
      s.a[1][q] = g.get(c, FY, p);
      s.a[2][q] = g.get(c, FZ, p);
    }
  }
  check(s.ctx, gbmd_upload_atoms(s.ctx, (int64_t)n, s.r[0].data(), s.r[1].data(), s.r[2].data(), s.v[0].data(),
                                 s.v[1].data(), s.v[2].data(), s.type.data(), s.id_now.data()),
        "gbmd_upload_atoms");
  check(s.ctx, gbmd_upload_state(s.ctx, s.r[0].data(), s.r[1].data(), s.r[2].data(), s.v[0].data(), s.v[1].data(),
                                 s.v[2].data(), s.a[0].data(), s.a[1].data(), s.a[2].data()),
        "gbmd_upload_state");
  record_layout(s);
  ++s.full_uploads;
  s.resident = true;
  s.grid_stale = false;
}

// push_f_v_r / push_f_v of verlet_first_half and verlet_second_half on the
// device's copy (exaNBody's push operators; formula
// push_vec3_2nd_order_xform_minimization.cpp L33-38).
template <class G>
void push_f_v_r(Session& s, G& g, double dt, double dt_scale) {
  apply_xform(s, g);
  make_resident(s, g);
  check(s.ctx, gbmd_push_f_v_r(s.ctx, dt, dt_scale), "gbmd_push_f_v_r");
  s.grid_stale = true;
}

template <class G>
void push_f_v(Session& s, G& g, double dt, double dt_scale) {
  apply_xform(s, g);
  make_resident(s, g);
  check(s.ctx, gbmd_push_f_v(s.ctx, dt, dt_scale), "gbmd_push_f_v");
  s.grid_stale = true;
}

// check_and_update_particles on the device's copy: rebuild when some atom
// moved more than skin/2.  Returns whether it rebuilt.
template <class G>
bool update_neighbors(Session& s, G& g) {
  apply_xform(s, g);
  make_resident(s, g);
  int rebuilt = 0;
  check(s.ctx, gbmd_update_neighbors(s.ctx, &rebuilt), "gbmd_update_neighbors");
  return rebuilt != 0;
}

// The device's state back into the grid's cells (resident mode): r, v, the
// accelerations into the f fields, ep and the virial when present.  Particles
// stay in the cells and slots of the upload (the library's rebinning is its
// own); a following move_particles re-bins them on the host if a run needs.
template <class G>
void sync_grid(Session& s, G& g, bool energy, bool virial) {
  if (!s.resident || !s.grid_stale) return;
  const size_t n = s.n;
  for (int d = 0; d < 3; ++d) {
    s.r[d].resize(n);
    s.v[d].resize(n);
    s.a[d].resize(n);
  }
  if (energy) s.ep.resize(n);
  const bool vir = virial && g.has_virial();
  if (vir) s.vir.resize(9 * n);
  check(s.ctx, gbmd_download(s.ctx, s.r[0].data(), s.r[1].data(), s.r[2].data(), s.v[0].data(), s.v[1].data(),
                             s.v[2].data(), s.a[0].data(), s.a[1].data(), s.a[2].data(),
                             energy ? s.ep.data() : nullptr, vir ? s.vir.data() : nullptr),
        "gbmd_download");
  check(s.ctx, gbmd_check_errors(s.ctx), "gbmd_check_errors");
  for (size_t k = 0; k < n; ++k) {
    const size_t c = s.cell[k], p = s.slot[k];
    g.set(c, RX, p, s.r[0][k] / s.scale[0]);
    g.set(c, RY, p, s.r[1][k] / s.scale[1]);
    g.set(c, RZ, p, s.r[2][k] / s.scale[2]);
    g.set(c, VX, p, s.v[0][k]);
    g.set(c, VY, p, s.v[1][k]);
    g.set(c, VZ, p, s.v[2][k]);
    g.set(c, FX, p, s.a[0][k]);
    g.set(c, FY, p, s.a[1][k]);
    g.set(c, FZ, p, s.a[2][k]);
    if (energy) g.set(c, EP, p, s.ep[k]);
    if (vir) g.set_virial(c, p, &s.vir[9 * k]);
  }
  s.grid_stale = false;
}

}  // namespace gb300
