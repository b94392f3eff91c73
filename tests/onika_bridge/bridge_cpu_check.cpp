// bridge_cpu_check.cpp -- the onika plugin's host logic
// (exastamp_gb300/onika/gb300_bridge.h) on the CPU, over a stand-in of the
// libgbmd entry points it calls (defined below, no device).  Test
// infrastructure for tests/test_bridge_cpu.py.
//
// The stand-in keeps the uploaded state in host arrays and records the box
// and the upload counts; its "forces" are a = -(r - centre) of the box it was
// given, so a wrong box or a wrong coordinate scale shows in the results.
// Checks (each failure prints a line and the program returns 1):
//   1  diagonal xform at creation: the box handed over is the grid bounds
//      times the scale; gathered positions are grid coordinates times it
//   2  per-call forces written back as f = m a; same layout: positions-only
//      upload; a reordered layout at the same count: full upload
//   3  resident steps: pushes on the device copy, sync_grid writes the
//      positions back divided by the scale
//   4  a changed xform between calls while the device copy is newer than the
//      grid: synced back with the old scale first, then the box and a full
//      upload with the new scale (grid coordinates unchanged)
//   5  a device error reported by gbmd_check_errors stops a force call
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "gb300_bridge.h"

// ---- stand-in of the libgbmd entry points the bridge calls ------------------
struct gbmd_context {
  double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
  int64_t n = 0;
  std::vector<double> r[3], v[3], a[3], ep;
  std::vector<uint8_t> type;
  std::vector<uint64_t> id;
  std::vector<double> masses;
  int set_box_calls = 0, full_uploads = 0, position_uploads = 0;
  int pending_error = 0;
};

extern "C" {
int gbmd_create(gbmd_context** ctx, int, void*) {
  *ctx = new gbmd_context();
  return GBMD_OK;
}
int gbmd_destroy(gbmd_context* c) {
  delete c;
  return GBMD_OK;
}
const char* gbmd_last_error(const gbmd_context*) { return "stand-in error"; }
int gbmd_set_box(gbmd_context* c, const double lo[3], const double hi[3], const int*) {
  for (int d = 0; d < 3; ++d) {
    c->lo[d] = lo[d];
    c->hi[d] = hi[d];
  }
  ++c->set_box_calls;
  return GBMD_OK;
}
int gbmd_set_species(gbmd_context* c, int ntypes, const double* m) {
  c->masses.assign(m, m + ntypes);
  return GBMD_OK;
}
int gbmd_upload_atoms(gbmd_context* c, int64_t n, const double* rx, const double* ry, const double* rz,
                      const double* vx, const double* vy, const double* vz, const uint8_t* type,
                      const uint64_t* id) {
  c->n = n;
  const double* rr[3] = {rx, ry, rz};
  const double* vv[3] = {vx, vy, vz};
  for (int d = 0; d < 3; ++d) {
    c->r[d].assign(rr[d], rr[d] + n);
    c->v[d].assign(vv[d], vv[d] + n);
    c->a[d].assign((size_t)n, 0.0);
  }
  c->type.assign(type, type + n);
  c->id.assign(id, id + n);
  c->ep.assign((size_t)n, 0.0);
  ++c->full_uploads;
  return GBMD_OK;
}
int gbmd_upload_positions(gbmd_context* c, const double* rx, const double* ry, const double* rz, const double*,
                          const double*, const double*) {
  const double* rr[3] = {rx, ry, rz};
  for (int d = 0; d < 3; ++d) c->r[d].assign(rr[d], rr[d] + c->n);
  ++c->position_uploads;
  return GBMD_OK;
}
int gbmd_upload_state(gbmd_context* c, const double* rx, const double* ry, const double* rz, const double* vx,
                      const double* vy, const double* vz, const double* ax, const double* ay, const double* az) {
  const double* p[9] = {rx, ry, rz, vx, vy, vz, ax, ay, az};
  for (int d = 0; d < 3; ++d) {
    c->r[d].assign(p[d], p[d] + c->n);
    c->v[d].assign(p[3 + d], p[3 + d] + c->n);
    c->a[d].assign(p[6 + d], p[6 + d] + c->n);
  }
  return GBMD_OK;
}
int gbmd_compute_forces(gbmd_context* c, int) {
  for (int d = 0; d < 3; ++d)
    for (int64_t i = 0; i < c->n; ++i) c->a[d][i] = -(c->r[d][i] - 0.5 * (c->lo[d] + c->hi[d]));
  for (int64_t i = 0; i < c->n; ++i) c->ep[i] = 1.0;
  return GBMD_OK;
}
int gbmd_check_errors(gbmd_context* c) {
  const int e = c->pending_error;
  c->pending_error = 0;
  return e;
}
int gbmd_download(gbmd_context* c, double* rx, double* ry, double* rz, double* vx, double* vy, double* vz,
                  double* ax, double* ay, double* az, double* ep, double* vir) {
  double* out[9] = {rx, ry, rz, vx, vy, vz, ax, ay, az};
  const std::vector<double>* src[9] = {&c->r[0], &c->r[1], &c->r[2], &c->v[0], &c->v[1],
                                       &c->v[2], &c->a[0], &c->a[1], &c->a[2]};
  for (int k = 0; k < 9; ++k)
    if (out[k]) std::memcpy(out[k], src[k]->data(), sizeof(double) * (size_t)c->n);
  if (ep) std::memcpy(ep, c->ep.data(), sizeof(double) * (size_t)c->n);
  if (vir) std::memset(vir, 0, sizeof(double) * 9 * (size_t)c->n);
  return GBMD_OK;
}
int gbmd_push_f_v_r(gbmd_context* c, double dt, double s) {
  const double h = dt * s;
  for (int d = 0; d < 3; ++d)
    for (int64_t i = 0; i < c->n; ++i) c->r[d][i] += c->v[d][i] * h + c->a[d][i] * h * h * 0.5;
  return GBMD_OK;
}
int gbmd_push_f_v(gbmd_context* c, double dt, double s) {
  for (int d = 0; d < 3; ++d)
    for (int64_t i = 0; i < c->n; ++i) c->v[d][i] += c->a[d][i] * dt * s;
  return GBMD_OK;
}
int gbmd_update_neighbors(gbmd_context*, int* rebuilt) {
  if (rebuilt) *rebuilt = 0;
  return GBMD_OK;
}
}

// ---- a small cell grid (no ghost layer needed by the checks) -----------------
struct Grid {
  struct Cell {
    std::vector<double> f[10];
    std::vector<uint8_t> type;
    std::vector<uint64_t> id;
    size_t size() const { return id.size(); }
  };
  std::vector<Cell> cells;
  std::vector<double> masses{1.0, 2.0};
  size_t inner_cells() const { return cells.size(); }
  size_t cell_index(size_t k) const { return k; }
  size_t cell_size(size_t c) const { return cells[c].size(); }
  double get(size_t c, gb300::Field f, size_t p) const { return cells[c].f[f][p]; }
  void set(size_t c, gb300::Field f, size_t p, double v) { cells[c].f[f][p] = v; }
  uint8_t type(size_t c, size_t p) const { return cells[c].type[p]; }
  uint64_t id(size_t c, size_t p) const { return cells[c].id[p]; }
  bool has_virial() const { return false; }
  void set_virial(size_t, size_t, const double*) {}
  double mass(int t) const { return masses[t]; }
};

static int failures = 0;
static void expect(bool ok, const char* what) {
  if (!ok) {
    std::printf("FAIL %s\n", what);
    ++failures;
  }
}
static bool near(double a, double b) { return std::fabs(a - b) <= 1e-12 * (1.0 + std::fabs(b)); }

int main() {
  // 2 cells x 3 atoms in grid coordinates of the box [0, 4) x [0, 2) x [0, 1)
  Grid g;
  g.cells.resize(2);
  uint64_t next_id = 100;
  for (int c = 0; c < 2; ++c)
    for (int p = 0; p < 3; ++p) {
      auto& cell = g.cells[c];
      const double q = 0.1 + 0.25 * (3 * c + p);
      const double vals[10] = {q, 0.5 * q, 0.25 * q, 0.01 * (p + 1), -0.02, 0.03, 0, 0, 0, 0};
      for (int k = 0; k < 10; ++k) cell.f[k].push_back(vals[k]);
      cell.type.push_back((uint8_t)(p % 2));
      cell.id.push_back(next_id++);
    }
  const double glo[3] = {0, 0, 0}, ghi[3] = {4, 2, 1};
  const int per[3] = {1, 1, 1};
  const double s1[3] = {1.5, 0.5, 2.0}, s2[3] = {1.25, 0.75, 2.5};
  try {
    gb300::Session s;
    gb300::ensure_context(s, nullptr, glo, ghi, per, g.masses, s1);
    gbmd_context* c = s.ctx;
    // 1
    for (int d = 0; d < 3; ++d) expect(c->lo[d] == glo[d] * s1[d] && c->hi[d] == ghi[d] * s1[d], "1 box scaled");
    // 2
    gb300::set_xform_scale(s, s1);
    gb300::compute_forces(s, g, true, false, 0);
    expect(c->full_uploads == 1 && c->position_uploads == 0, "2 first call uploads every field");
    for (int64_t i = 0; i < c->n; ++i) {
      const size_t cc = s.cell[(size_t)i], p = s.slot[(size_t)i];
      for (int d = 0; d < 3; ++d) expect(c->r[d][i] == g.get(cc, (gb300::Field)(gb300::RX + d), p) * s1[d],
                                         "2 physical positions uploaded");
      const double m = g.mass(g.type(cc, p));
      expect(near(g.get(cc, gb300::FX, p), m * c->a[0][i]), "2 f = m a written back");
    }
    gb300::compute_forces(s, g, true, false, 0);
    expect(c->full_uploads == 1 && c->position_uploads == 1, "2 same layout: positions only");
    std::swap(g.cells[0], g.cells[1]);
    gb300::compute_forces(s, g, true, false, 0);
    expect(c->full_uploads == 2, "2 reordered layout at the same count: full upload");
    // 3: resident steps (f fields taken as accelerations)
    gb300::push_f_v_r(s, g, 0.1, 1.0);
    expect(c->full_uploads == 3, "3 whole-step mode uploads the state once");
    gb300::push_f_v(s, g, 0.1, 0.5);
    gb300::sync_grid(s, g, false, false);
    for (int64_t i = 0; i < c->n; ++i) {
      const size_t cc = s.cell[(size_t)i], p = s.slot[(size_t)i];
      for (int d = 0; d < 3; ++d)
        expect(g.get(cc, (gb300::Field)(gb300::RX + d), p) == c->r[d][i] / s1[d], "3 positions back / scale");
      expect(g.get(cc, gb300::VX, p) == c->v[0][i], "3 velocities back unscaled");
    }
    // 4: device copy newer than the grid, then the xform changes
    gb300::push_f_v_r(s, g, 0.1, 1.0);
    std::vector<double> phys_old[3];
    for (int d = 0; d < 3; ++d) phys_old[d] = c->r[d];
    const int boxes = c->set_box_calls, full = c->full_uploads;
    gb300::set_xform_scale(s, s2);
    gb300::update_neighbors(s, g);
    expect(c->set_box_calls == boxes + 1, "4 new box");
    for (int d = 0; d < 3; ++d) expect(c->lo[d] == glo[d] * s2[d] && c->hi[d] == ghi[d] * s2[d], "4 box rescaled");
    expect(c->full_uploads == full + 1, "4 full upload after the rescale");
    for (int64_t i = 0; i < c->n; ++i)
      for (int d = 0; d < 3; ++d)
        expect(c->r[d][i] == (phys_old[d][i] / s1[d]) * s2[d], "4 old state synced, new scale applied");
    // 5
    c->pending_error = GBMD_ERR_NONFINITE;
    bool thrown = false;
    try {
      s.resident = false;
      gb300::compute_forces(s, g, true, false, 0);
    } catch (const gb300::Error&) {
      thrown = true;
    }
    expect(thrown, "5 device error stops the force call");
    bool refused = false;
    try {
      const double bad[3] = {1.0, -1.0, 1.0};
      gb300::set_xform_scale(s, bad);
    } catch (const gb300::Error&) {
      refused = true;
    }
    expect(refused, "5 non-positive scale refused");
  } catch (const gb300::Error& e) {
    std::printf("FAIL unexpected error: %s\n", e.what());
    return 1;
  }
  if (failures) return 1;
  std::printf("ok\n");
  return 0;
}
