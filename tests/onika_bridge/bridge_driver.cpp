// bridge_driver.cpp -- drives the onika plugin's host logic
// (exastamp_gb300/onika/gb300_bridge.h) over a fake exaNBody cell grid,
// through libgbmd on the GPU.  Test infrastructure for
// tests/test_gpu_onika_bridge.py, which writes the input and checks the
// output against the FP64 oracle.
//
//   bridge_driver <input.bin> <output.bin> [sx sy sz [tx ty tz]]
//
// With sx sy sz the domain has the diagonal xform diag(sx, sy, sz): the input
// positions and bounds are grid coordinates, the physical ones are scaled.
// With tx ty tz the xform becomes diag(tx, ty, tz) half-way through phase D
// (before that step's push_f_v_r), as a deformation run changes it.
//
// Input (little endian): int64 n, ntypes, nsteps, ncell[3]; double lo[3],
// hi[3], epsilon, sigma, rcut, skin, dt; double masses[ntypes];
// double x, y, z, vx, vy, vz [n]; uint8 type[n]; uint64 id[n].
// The grid has one ghost layer (empty cells) around ncell^3 inner cells;
// each atom goes to the inner cell of its position, in input order.
//
// Phases (LJ, FP64 precision, energies and virials on):
//   A  per-call forces of the input state
//   B  every position moved by a small seeded offset, same layout
//      (positions-only upload)
//   C  move_particles-like reordering at constant count: each cell's
//      particles reversed, every 5th particle of a cell moved to the next
//      cell (full upload, new layout)
//   D  whole-step run from C's state: the f fields turned into accelerations,
//      then nsteps of push_f_v_r, push_f_v, update_neighbors, forces,
//      push_f_v on the device, then sync_grid
// Output: for each phase the counters (full uploads, position uploads) and
// one record per particle in grid order: id, r[3], v[3], f[3], ep, vir[9].
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "gb300_bridge.h"

namespace {

struct FakeGrid {
  int64_t nc[3] = {0, 0, 0}, dims[3] = {0, 0, 0};
  struct Cell {
    std::vector<double> f[10];
    std::vector<uint8_t> type;
    std::vector<uint64_t> id;
    std::vector<double> vir;
    size_t size() const { return id.size(); }
    void push(const double* v10, uint8_t t, uint64_t i) {
      for (int k = 0; k < 10; ++k) f[k].push_back(v10[k]);
      type.push_back(t);
      id.push_back(i);
      for (int q = 0; q < 9; ++q) vir.push_back(0.0);
    }
  };
  std::vector<Cell> cells;
  std::vector<size_t> inner;
  std::vector<double> masses;

  void init(const int64_t n3[3]) {
    for (int d = 0; d < 3; ++d) {
      nc[d] = n3[d];
      dims[d] = n3[d] + 2;  // one ghost layer
    }
    cells.assign((size_t)(dims[0] * dims[1] * dims[2]), Cell{});
    inner.clear();
    for (int64_t k = 1; k <= nc[2]; ++k)
      for (int64_t j = 1; j <= nc[1]; ++j)
        for (int64_t i = 1; i <= nc[0]; ++i) inner.push_back((size_t)((k * dims[1] + j) * dims[0] + i));
  }
  // grid-view interface of gb300_bridge.h
  size_t inner_cells() const { return inner.size(); }
  size_t cell_index(size_t k) const { return inner[k]; }
  size_t cell_size(size_t c) const { return cells[c].size(); }
  double get(size_t c, gb300::Field f, size_t p) const { return cells[c].f[f][p]; }
  void set(size_t c, gb300::Field f, size_t p, double v) { cells[c].f[f][p] = v; }
  uint8_t type(size_t c, size_t p) const { return cells[c].type[p]; }
  uint64_t id(size_t c, size_t p) const { return cells[c].id[p]; }
  bool has_virial() const { return true; }
  void set_virial(size_t c, size_t p, const double v[9]) { std::memcpy(&cells[c].vir[9 * p], v, 9 * sizeof(double)); }
  double mass(int t) const { return masses[t]; }
};

template <class T>
bool rd(FILE* f, T* p, size_t n) {
  return std::fread(p, sizeof(T), n, f) == n;
}

void dump(FILE* out, const FakeGrid& g, const gb300::Session& s) {
  const int64_t cnt[2] = {s.full_uploads, s.position_uploads};
  std::fwrite(cnt, sizeof(int64_t), 2, out);
  for (size_t k = 0; k < g.inner_cells(); ++k) {
    const auto& c = g.cells[g.cell_index(k)];
    for (size_t p = 0; p < c.size(); ++p) {
      double rec[20];
      std::memcpy(&rec[0], &c.id[p], sizeof(double));  // id bits
      for (int q = 0; q < 10; ++q) rec[1 + q] = c.f[q][p];
      for (int q = 0; q < 9; ++q) rec[11 + q] = c.vir[9 * p + q];
      std::fwrite(rec, sizeof(double), 20, out);
    }
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3 && argc != 6 && argc != 9) {
    std::fprintf(stderr, "usage: bridge_driver input.bin output.bin [sx sy sz [tx ty tz]]\n");
    return 2;
  }
  double scale1[3] = {1.0, 1.0, 1.0}, scale2[3] = {1.0, 1.0, 1.0};
  for (int d = 0; d < 3 && argc >= 6; ++d) scale1[d] = std::strtod(argv[3 + d], nullptr);
  for (int d = 0; d < 3 && argc == 9; ++d) scale2[d] = std::strtod(argv[6 + d], nullptr);
  FILE* in = std::fopen(argv[1], "rb");
  if (!in) return 2;
  int64_t hdr[6];
  double prm[11];
  if (!rd(in, hdr, 6) || !rd(in, prm, 11)) return 2;
  const int64_t n = hdr[0], ntypes = hdr[1], nsteps = hdr[2];
  const double *lo = prm, *hi = prm + 3;
  const double eps = prm[6], sig = prm[7], rcut = prm[8], skin = prm[9], dt = prm[10];
  FakeGrid g;
  g.masses.resize((size_t)ntypes);
  std::vector<double> a[6];
  for (auto& v : a) v.resize((size_t)n);
  std::vector<uint8_t> type((size_t)n);
  std::vector<uint64_t> id((size_t)n);
  bool ok = rd(in, g.masses.data(), (size_t)ntypes);
  for (auto& v : a) ok = ok && rd(in, v.data(), (size_t)n);
  ok = ok && rd(in, type.data(), (size_t)n) && rd(in, id.data(), (size_t)n);
  std::fclose(in);
  if (!ok) return 2;
  g.init(hdr + 3);
  for (int64_t q = 0; q < n; ++q) {
    int64_t c[3];
    for (int d = 0; d < 3; ++d) {
      const double h = (hi[d] - lo[d]) / (double)g.nc[d];
      c[d] = (int64_t)std::floor(((d == 0 ? a[0] : d == 1 ? a[1] : a[2])[q] - lo[d]) / h);
      c[d] = c[d] < 0 ? 0 : (c[d] >= g.nc[d] ? g.nc[d] - 1 : c[d]);
    }
    const size_t cell = (size_t)(((c[2] + 1) * g.dims[1] + (c[1] + 1)) * g.dims[0] + (c[0] + 1));
    const double v10[10] = {a[0][q], a[1][q], a[2][q], a[3][q], a[4][q], a[5][q], 0, 0, 0, 0};
    g.cells[cell].push(v10, type[q], id[q]);
  }
  FILE* out = std::fopen(argv[2], "wb");
  if (!out) return 2;
  try {
    gb300::Session s;
    const int per[3] = {1, 1, 1};
    gb300::ensure_context(s, nullptr, lo, hi, per, g.masses, argc >= 6 ? scale1 : nullptr);
    gb300::check(s.ctx, gbmd_set_lj(s.ctx, eps, sig, rcut), "gbmd_set_lj");
    gb300::check(s.ctx, gbmd_set_skin(s.ctx, skin), "gbmd_set_skin");
    gb300::check(s.ctx, gbmd_set_precision(s.ctx, GBMD_PRECISION_FP64), "gbmd_set_precision");
    // A
    gb300::compute_forces(s, g, true, true, 0);
    dump(out, g, s);
    // B
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> u(-0.02, 0.02);
    for (size_t k = 0; k < g.inner_cells(); ++k) {
      auto& c = g.cells[g.cell_index(k)];
      for (size_t p = 0; p < c.size(); ++p)
        for (int d = 0; d < 3; ++d) c.f[d][p] += u(rng);
    }
    gb300::compute_forces(s, g, true, true, 0);
    dump(out, g, s);
    // C
    std::vector<FakeGrid::Cell> moved(g.cells.size());
    for (size_t k = 0; k < g.inner_cells(); ++k) {
      const size_t ci = g.cell_index(k), cn = g.cell_index((k + 1) % g.inner_cells());
      const auto& c = g.cells[ci];
      for (size_t p = c.size(); p-- > 0;) {
        double v10[10];
        for (int q = 0; q < 10; ++q) v10[q] = c.f[q][p];
        (p % 5 == 0 ? moved[cn] : moved[ci]).push(v10, c.type[p], c.id[p]);
      }
    }
    g.cells.swap(moved);
    gb300::compute_forces(s, g, true, true, 0);
    dump(out, g, s);
    // D: the grid's force_to_accel, then the whole step on the device
    for (size_t k = 0; k < g.inner_cells(); ++k) {
      auto& c = g.cells[g.cell_index(k)];
      for (size_t p = 0; p < c.size(); ++p)
        for (int d = 0; d < 3; ++d) c.f[gb300::FX + d][p] /= g.masses[c.type[p]];
    }
    for (int64_t st = 0; st < nsteps; ++st) {
      if (argc == 9 && st == nsteps / 2) gb300::set_xform_scale(s, scale2);
      gb300::push_f_v_r(s, g, dt, 1.0);
      gb300::push_f_v(s, g, dt, 0.5);
      gb300::update_neighbors(s, g);
      gb300::compute_forces(s, g, st + 1 == nsteps, false, 0);
      gb300::push_f_v(s, g, dt, 0.5);
    }
    gb300::sync_grid(s, g, true, false);
    dump(out, g, s);
  } catch (const gb300::Error& e) {
    std::fprintf(stderr, "%s\n", e.what());
    std::fclose(out);
    return 1;
  }
  std::fclose(out);
  return 0;
}
