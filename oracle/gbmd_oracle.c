/*
 * gbmd_oracle.c -- CPU FP64 restatement of exaStamp's MD hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the correctness oracle and the timed CPU baseline
 * for the GB300 kernels.  The product path never links or calls this file.
 *
 * Build: gcc -O3 -fopenmp -ffp-contract=off -fPIC -shared (see oracle/oracle.py).
 * -ffp-contract=off matters: the neighbour test d2 <= R^2 must round exactly
 * like the GPU list builder, which evaluates it with explicit _rn intrinsics.
 *
 * Reference files restated (paths inside the exaStamp tree):
 *   LJ pair      src/potential/pair_potentials/lennard_jones/include/exaStamp/
 *                potential/pair_potentials/lennard_jones/lennard_jones.h L41-50
 *   LJ per atom  src/potential/pair_potential_template/force_op_impl2.hxx L22-78
 *   LJ ecut      src/potential/pair_potential_template/pair_potential_impl.hxx L489-498
 *   LJ multi     src/potential/pair_potential_template/pair_potential_force_op_multiparam.h L75-118
 *   EAM spline   src/potential/eam_potentials/eam_alloy/eam_alloy.cpp L29-58
 *   EAM lookups  src/potential/eam_potentials/eam_alloy/eam_alloy.h L198-313
 *   EAM passes   src/potential/eam_potential_template/eam_force_op_multimat.h L114-343
 *   mono-material EAM passes  src/potential/eam_potential_template/eam_force_op_singlemat.h L39-171
 *   johnson      src/potential/eam_potentials/johnson/johnson.h L55-176
 *   sutton_chen  src/potential/eam_potentials/sutton_chen/sutton_chen.h L40-66
 *   zero / accel src/compute/zero_force_energy.cu L38-47, src/compute/force_to_accel.cu L42-48
 *   push         src/numerical_schemes/push_vec3_2nd_order_xform_minimization.cpp L33-38, L116-149
 *   thermo       src/thermo_state/simulation_thermodynamic_state.cpp L101-163
 *   pair decode  src/debug/atom_neighbors_stats.cpp L169-209 (d2 formula and d2 <= R^2 test)
 */
#include "gbmd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Cell grid                                                                 */
/* ------------------------------------------------------------------------ */

/* Cells per dimension: the largest count whose edge stays >= R (with a 2^-40
 * relative margin so that binning round-off can never hide a pair), capped at
 * 1024 so that cell coordinates pack into 10 bits on the GPU. */
int orc_grid_dims(const double lo[3], const double hi[3], double R, int nc[3]) {
  for (int d = 0; d < 3; ++d) {
    double L = hi[d] - lo[d];
    if (!(L > 0.0) || !(R > 0.0)) return -1;
    double q = floor(L / (R * (1.0 + 0x1p-40)));
    if (q < 1.0) return -2; /* box thinner than the neighbour radius */
    if (q > 1024.0) q = 1024.0;
    nc[d] = (int)q;
  }
  return 0;
}

/* Periodic wrap into [lo, hi), one image at most (exaNBody move_particles
 * contract; atoms move far less than a box length between rebuilds).
 * Returns how many atoms are still outside afterwards ("lost atoms"). */
int64_t orc_wrap(int64_t n, double* x, double* y, double* z, const double lo[3], const double hi[3]) {
  int64_t lost = 0;
  double* r[3] = {x, y, z};
  for (int d = 0; d < 3; ++d) {
    const double L = hi[d] - lo[d];
    double* a = r[d];
#pragma omp parallel for schedule(static) reduction(+ : lost)
    for (int64_t i = 0; i < n; ++i) {
      double v = a[i];
      if (v < lo[d]) v += L;
      else if (v >= hi[d]) v -= L;
      if (v < lo[d] || v >= hi[d]) ++lost;
      a[i] = v;
    }
  }
  return lost;
}

static inline int cell_coord(double v, double lo, double inv_h, int nc) {
  int c = (int)((v - lo) * inv_h);
  if (c < 0) c = 0;
  if (c > nc - 1) c = nc - 1;
  return c;
}

typedef struct {
  int nc[3];
  int64_t ncells;
  int64_t* start; /* ncells+1 */
  int64_t* atoms; /* n, sorted by (cell, id, index) */
  int32_t* cell_of; /* n */
} orc_grid;

static int grid_build(orc_grid* g, int64_t n, const double* x, const double* y, const double* z,
                      const uint64_t* id, const double lo[3], const double hi[3], double R) {
  if (orc_grid_dims(lo, hi, R, g->nc) != 0) return -1;
  double inv_h[3];
  for (int d = 0; d < 3; ++d) inv_h[d] = (double)g->nc[d] / (hi[d] - lo[d]);
  g->ncells = (int64_t)g->nc[0] * g->nc[1] * g->nc[2];
  g->start = (int64_t*)calloc((size_t)g->ncells + 1, sizeof(int64_t));
  g->atoms = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  g->cell_of = (int32_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    int cx = cell_coord(x[i], lo[0], inv_h[0], g->nc[0]);
    int cy = cell_coord(y[i], lo[1], inv_h[1], g->nc[1]);
    int cz = cell_coord(z[i], lo[2], inv_h[2], g->nc[2]);
    g->cell_of[i] = (int32_t)(((int64_t)cz * g->nc[1] + cy) * g->nc[0] + cx);
  }
  for (int64_t i = 0; i < n; ++i) g->start[g->cell_of[i] + 1]++;
  for (int64_t c = 0; c < g->ncells; ++c) g->start[c + 1] += g->start[c];
  int64_t* fill = (int64_t*)malloc((size_t)g->ncells * sizeof(int64_t));
  memcpy(fill, g->start, (size_t)g->ncells * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) g->atoms[fill[g->cell_of[i]]++] = i;
  free(fill);
  /* canonical order inside a cell: ascending id, then ascending input index */
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t c = 0; c < g->ncells; ++c) {
    int64_t b = g->start[c], e = g->start[c + 1];
    for (int64_t k = b + 1; k < e; ++k) {
      int64_t a = g->atoms[k];
      int64_t m = k - 1;
      while (m >= b) {
        int64_t o = g->atoms[m];
        int later = id ? (id[o] > id[a] || (id[o] == id[a] && o > a)) : (o > a);
        if (!later) break;
        g->atoms[m + 1] = o;
        --m;
      }
      g->atoms[m + 1] = a;
    }
  }
  return 0;
}

static void grid_free(orc_grid* g) {
  free(g->start);
  free(g->atoms);
  free(g->cell_of);
}

/* d2 of the pair (i, image n of j), no FMA: the reference's pair-decode
 * formula (atom_neighbors_stats.cpp L201-204) on ghost coordinates x_j + n*L. */
static inline double pair_d2(const double* x, const double* y, const double* z, int64_t i, int64_t j,
                             const int n[3], const double L[3], double* dx, double* dy, double* dz) {
  const double sx = (double)n[0] * L[0], sy = (double)n[1] * L[1], sz = (double)n[2] * L[2];
  *dx = (x[j] + sx) - x[i];
  *dy = (y[j] + sy) - y[i];
  *dz = (z[j] + sz) - z[i];
  return *dx * *dx + *dy * *dy + *dz * *dz;
}

/* Visit the 27-cell stencil of atom i in canonical order: stencil code
 * s = (dz+1)*9 + (dy+1)*3 + (dx+1) ascending, then the cell's atoms in
 * (id, index) order.  The image shift follows from wrapping the stencil cell. */
static int64_t visit_atom(const orc_grid* g, int64_t i, const double* x, const double* y,
                          const double* z, const double L[3], double R2, int32_t* nbr, int8_t* img) {
  const int c = g->cell_of[i];
  const int cx = c % g->nc[0], cy = (c / g->nc[0]) % g->nc[1], cz = c / (g->nc[0] * g->nc[1]);
  int64_t cnt = 0;
  for (int s = 0; s < 27; ++s) {
    const int d[3] = {s % 3 - 1, (s / 3) % 3 - 1, s / 9 - 1};
    const int cc[3] = {cx + d[0], cy + d[1], cz + d[2]};
    int n[3], w[3];
    for (int k = 0; k < 3; ++k) {
      n[k] = cc[k] < 0 ? -1 : (cc[k] >= g->nc[k] ? 1 : 0);
      w[k] = cc[k] - n[k] * g->nc[k];
    }
    const int64_t cj = ((int64_t)w[2] * g->nc[1] + w[1]) * g->nc[0] + w[0];
    const int self_image = (n[0] == 0 && n[1] == 0 && n[2] == 0);
    for (int64_t k = g->start[cj]; k < g->start[cj + 1]; ++k) {
      const int64_t j = g->atoms[k];
      if (j == i && self_image) continue;
      double dx, dy, dz;
      const double d2 = pair_d2(x, y, z, i, j, n, L, &dx, &dy, &dz);
      if (d2 <= R2) {
        if (nbr) {
          nbr[cnt] = (int32_t)j;
          img[3 * cnt + 0] = (int8_t)n[0];
          img[3 * cnt + 1] = (int8_t)n[1];
          img[3 * cnt + 2] = (int8_t)n[2];
        }
        ++cnt;
      }
    }
  }
  return cnt;
}

/* Full (non-Newton) neighbour list within R = rcut + skin, CSR by atom.
 * Restates the pair set of exaNBody's chunk_neighbors with chunk_size 1, as
 * decoded by atom_neighbors_stats.cpp L169-228.  Returns the total number of
 * pairs; nbr/img are written only when cap is large enough (else call again). */
int64_t orc_build_neighbors(int64_t n, const double* x, const double* y, const double* z,
                            const uint64_t* id, const double lo[3], const double hi[3], double R,
                            int64_t* offsets, int64_t cap, int32_t* nbr, int8_t* img) {
  return orc_build_neighbors_first(n, n, x, y, z, id, lo, hi, R, offsets, cap, nbr, img);
}

/* The same list for the first nlist atoms only (their neighbours taken among
 * all n): a bounded sample of a large system's pair set. */
int64_t orc_build_neighbors_first(int64_t n, int64_t nlist, const double* x, const double* y, const double* z,
                                  const uint64_t* id, const double lo[3], const double hi[3], double R,
                                  int64_t* offsets, int64_t cap, int32_t* nbr, int8_t* img) {
  if (nlist < 0 || nlist > n) return -1;
  orc_grid g;
  if (grid_build(&g, n, x, y, z, id, lo, hi, R) != 0) return -1;
  const double L[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  const double R2 = R * R;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < nlist; ++i) offsets[i + 1] = visit_atom(&g, i, x, y, z, L, R2, NULL, NULL);
  offsets[0] = 0;
  for (int64_t i = 0; i < nlist; ++i) offsets[i + 1] += offsets[i];
  const int64_t total = offsets[nlist];
  if (nbr && total <= cap) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < nlist; ++i) visit_atom(&g, i, x, y, z, L, R2, nbr + offsets[i], img + 3 * offsets[i]);
  }
  grid_free(&g);
  return total;
}

/* O(N^2 * 27) all-image pair enumeration; independent check of the cell list. */
int64_t orc_brute_pairs(int64_t n, const double* x, const double* y, const double* z,
                        const double lo[3], const double hi[3], double R, int64_t cap,
                        int32_t* pi, int32_t* pj, int8_t* img) {
  const double L[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  const double R2 = R * R;
  int64_t cnt = 0;
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = 0; j < n; ++j)
      for (int s = 0; s < 27; ++s) {
        const int nn[3] = {s % 3 - 1, (s / 3) % 3 - 1, s / 9 - 1};
        if (i == j && nn[0] == 0 && nn[1] == 0 && nn[2] == 0) continue;
        double dx, dy, dz;
        if (pair_d2(x, y, z, i, j, nn, L, &dx, &dy, &dz) <= R2) {
          if (cnt < cap) {
            pi[cnt] = (int32_t)i;
            pj[cnt] = (int32_t)j;
            img[3 * cnt] = (int8_t)nn[0];
            img[3 * cnt + 1] = (int8_t)nn[1];
            img[3 * cnt + 2] = (int8_t)nn[2];
          }
          ++cnt;
        }
      }
  return cnt;
}

/* ------------------------------------------------------------------------ */
/* Lennard-Jones                                                             */
/* ------------------------------------------------------------------------ */

/* lennard_jones.h L41-50: e = 4 eps (s12 - s6), de = dE/dr. */
void orc_lj_pair(double epsilon, double sigma, double r, double* e, double* de) {
  const double ratio = sigma / r;
  const double ratio2 = ratio * ratio;
  const double ratio6 = ratio2 * ratio2 * ratio2;
  const double ratio12 = ratio6 * ratio6;
  *e = 4. * epsilon * (ratio12 - ratio6);
  *de = (-24. * epsilon * (2. * ratio12 - ratio6)) / r;
}

/* pair_potential_impl.hxx L489-498: ecut = e(rcut), 0 when rcut <= 0. */
double orc_lj_energy_cut(double epsilon, double sigma, double rcut) {
  double e = 0.0, de = 0.0;
  if (rcut > 0.0) orc_lj_pair(epsilon, sigma, rcut, &e, &de);
  return e;
}

static inline void add_vir(double* v, double fx, double fy, double fz, double dx, double dy, double dz) {
  /* tensor(fe, dr) * -0.5, row-major m11..m33 */
  v[0] += fx * dx * -0.5; v[1] += fx * dy * -0.5; v[2] += fx * dz * -0.5;
  v[3] += fy * dx * -0.5; v[4] += fy * dy * -0.5; v[5] += fy * dz * -0.5;
  v[6] += fz * dx * -0.5; v[7] += fz * dy * -0.5; v[8] += fz * dz * -0.5;
}

/* One in-cutoff pair of lj_compute_force's per-atom loop
 * (force_op_impl2.hxx L33-68): e -= ecut, de /= r, fe = de * dr, f += fe,
 * ep += e / 2, virial += (fe x dr) * -1/2.  acc = {fx, fy, fz, ep, vir[9]}. */
static inline void lj_accumulate(double epsilon, double sigma, double ecut, double dx, double dy, double dz,
                                 double d2, double* acc) {
  const double r = sqrt(d2);
  double e, de;
  orc_lj_pair(epsilon, sigma, r, &e, &de);
  e -= ecut;
  de /= r;
  const double fex = de * dx, fey = de * dy, fez = de * dz;
  acc[0] += fex; acc[1] += fey; acc[2] += fez;
  acc[3] += .5 * e;
  add_vir(acc + 4, fex, fey, fez, dx, dy, dz);
}

/* force_op_impl2.hxx L22-78 on one atom's pair buffer (drx, dry, drz, d2 of
 * its n in-cutoff neighbours, as the reference's ComputePairBuffer2 holds
 * them): out = {ep, fx, fy, fz, vir[9]}, each summed in buffer order. */
void orc_lj_atom_buffer(double epsilon, double sigma, double ecut, int n, const double* drx, const double* dry,
                        const double* drz, const double* d2, double* out) {
  double acc[13] = {0};
  for (int k = 0; k < n; ++k) lj_accumulate(epsilon, sigma, ecut, drx[k], dry[k], drz[k], d2[k], acc);
  out[0] = acc[3];
  out[1] = acc[0]; out[2] = acc[1]; out[3] = acc[2];
  for (int q = 0; q < 9; ++q) out[4 + q] = acc[4 + q];
}

/* lj_compute_force per atom (force_op_impl2.hxx L22-78) over the list pairs
 * with d2 <= rcut^2 (the traversal's rcut_max filter).  Zeroes first
 * (zero_force_energy), so outputs are the force on each atom, its half-pair
 * energy sum and its virial. */
void orc_lj_force(int64_t n, const double* x, const double* y, const double* z,
                  const int64_t* off, const int32_t* nbr, const int8_t* img, const double L[3],
                  const orc_lj_params* p, double* fx, double* fy, double* fz, double* ep, double* vir) {
  const double ecut = orc_lj_energy_cut(p->epsilon, p->sigma, p->rcut);
  const double rc2 = p->rcut * p->rcut;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    double acc[13] = {0};
    for (int64_t k = off[i]; k < off[i + 1]; ++k) {
      const int nn[3] = {img[3 * k], img[3 * k + 1], img[3 * k + 2]};
      double dx, dy, dz;
      const double d2 = pair_d2(x, y, z, i, nbr[k], nn, L, &dx, &dy, &dz);
      if (!(d2 <= rc2)) continue;
      lj_accumulate(p->epsilon, p->sigma, ecut, dx, dy, dz, d2, acc);
    }
    fx[i] = acc[0]; fy[i] = acc[1]; fz[i] = acc[2];
    if (ep) ep[i] = acc[3];
    if (vir) for (int q = 0; q < 9; ++q) vir[9 * i + q] = acc[4 + q];
  }
}

/* lj_multi_force (pair_potential_force_op_multiparam.h L75-118): traversal
 * filter d2 <= rcut_max^2, then per type pair r <= rcut_pair with that pair's
 * (eps, sigma) and ecut = e_pair(rcut_pair). */
void orc_lj_multi_force(int64_t n, const double* x, const double* y, const double* z, const uint8_t* type,
                        const int64_t* off, const int32_t* nbr, const int8_t* img, const double L[3],
                        const orc_lj_multi_params* p, double* fx, double* fy, double* fz, double* ep,
                        double* vir) {
  const int nt = p->ntypes;
  double* ecut = (double*)malloc(sizeof(double) * nt * nt);
  for (int a = 0; a < nt * nt; ++a) ecut[a] = orc_lj_energy_cut(p->epsilon[a], p->sigma[a], p->rcut[a]);
  const double rc2 = p->rcut_max * p->rcut_max;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    double acc[13] = {0};
    const int ta = type[i];
    for (int64_t k = off[i]; k < off[i + 1]; ++k) {
      const int nn[3] = {img[3 * k], img[3 * k + 1], img[3 * k + 2]};
      double dx, dy, dz;
      const int64_t j = nbr[k];
      const double d2 = pair_d2(x, y, z, i, j, nn, L, &dx, &dy, &dz);
      if (!(d2 <= rc2)) continue;
      const int pid = ta * nt + type[j];
      if (sqrt(d2) <= p->rcut[pid]) lj_accumulate(p->epsilon[pid], p->sigma[pid], ecut[pid], dx, dy, dz, d2, acc);
    }
    fx[i] = acc[0]; fy[i] = acc[1]; fz[i] = acc[2];
    if (ep) ep[i] = acc[3];
    if (vir) for (int q = 0; q < 9; ++q) vir[9 * i + q] = acc[4 + q];
  }
  free(ecut);
}

/* All-image direct LJ sum (no list, no cells): independent check of the
 * list-based path.  Returns the total energy (sum of per-atom half-pairs). */
double orc_lj_direct(int64_t n, const double* x, const double* y, const double* z, const double lo[3],
                     const double hi[3], const orc_lj_params* p, double* fx, double* fy, double* fz) {
  const double L[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  const double ecut = orc_lj_energy_cut(p->epsilon, p->sigma, p->rcut);
  const double rc2 = p->rcut * p->rcut;
  double etot = 0.0;
  int reach[3];
  for (int d = 0; d < 3; ++d) reach[d] = (int)ceil(p->rcut / L[d]) + 1;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : etot)
  for (int64_t i = 0; i < n; ++i) {
    double _fx = 0., _fy = 0., _fz = 0.;
    for (int64_t j = 0; j < n; ++j)
      for (int a = -reach[0]; a <= reach[0]; ++a)
        for (int b = -reach[1]; b <= reach[1]; ++b)
          for (int c = -reach[2]; c <= reach[2]; ++c) {
            if (i == j && a == 0 && b == 0 && c == 0) continue;
            const int nn[3] = {a, b, c};
            double dx, dy, dz;
            const double d2 = pair_d2(x, y, z, i, j, nn, L, &dx, &dy, &dz);
            if (!(d2 <= rc2)) continue;
            const double r = sqrt(d2);
            double e, de;
            orc_lj_pair(p->epsilon, p->sigma, r, &e, &de);
            e -= ecut;
            de /= r;
            _fx += de * dx; _fy += de * dy; _fz += de * dz;
            etot += 0.5 * e;
          }
    fx[i] = _fx; fy[i] = _fy; fz[i] = _fz;
  }
  return etot;
}

/* ------------------------------------------------------------------------ */
/* EAM alloy                                                                 */
/* ------------------------------------------------------------------------ */

/* eam_alloy.cpp L29-58 (LAMMPS array2spline): f[1..n] -> 7 coefficients per
 * knot; coefficients 0-2 give the derivative, 3-6 the value. spline is
 * (n+1) x 8 doubles, knot 0 left zero. */
void orc_eam_spline(int n, double delta, const double* f, double* spline) {
#define S(m, k) spline[(size_t)(m) * 8 + (k)]
  memset(spline, 0, sizeof(double) * 8 * (size_t)(n + 1));
  for (int m = 1; m <= n; m++) S(m, 6) = f[m];
  S(1, 5) = S(2, 6) - S(1, 6);
  S(2, 5) = 0.5 * (S(3, 6) - S(1, 6));
  S(n - 1, 5) = 0.5 * (S(n, 6) - S(n - 2, 6));
  S(n, 5) = S(n, 6) - S(n - 1, 6);
  for (int m = 3; m <= n - 2; m++)
    S(m, 5) = ((S(m - 2, 6) - S(m + 2, 6)) + 8.0 * (S(m + 1, 6) - S(m - 1, 6))) / 12.0;
  for (int m = 1; m <= n - 1; m++) {
    S(m, 4) = 3.0 * (S(m + 1, 6) - S(m, 6)) - 2.0 * S(m, 5) - S(m + 1, 5);
    S(m, 3) = S(m, 5) + S(m + 1, 5) - 2.0 * (S(m + 1, 6) - S(m, 6));
  }
  S(n, 4) = 0.0;
  S(n, 3) = 0.0;
  for (int m = 1; m <= n; m++) {
    S(m, 2) = S(m, 5) / delta;
    S(m, 1) = 2.0 * S(m, 4) / delta;
    S(m, 0) = 3.0 * S(m, 3) / delta;
  }
#undef S
}

static inline int z2r_index(int a, int b) {
  /* eam_alloy.h L113-132: irow >= icol, n = irow*(irow+1)/2 + icol */
  int irow = a > b ? a : b, icol = a > b ? b : a;
  return irow * (irow + 1) / 2 + icol;
}

static inline void r_knot(const orc_eam_tables* t, double r, int* m, double* p) {
  double pp = r * t->rdr + 1.0;
  int mm = (int)pp;
  if (mm > t->nr - 1) mm = t->nr - 1;
  pp -= mm;
  if (pp > 1.0) pp = 1.0;
  *m = mm;
  *p = pp;
}

/* eam_alloy_rho_noderiv (eam_alloy.h L198-220): density contributed at
 * distance r by an atom of element `itype` (the first type argument selects
 * the rhor table; SymRhoOp passes the neighbour's type first, L156). */
double orc_eam_rho(const orc_eam_tables* t, double r, int itype, int jtype) {
  (void)jtype;
  int m;
  double p;
  r_knot(t, r, &m, &p);
  const double* c = t->rhor + ((size_t)itype * (t->nr + 1) + m) * 8;
  return ((c[3] * p + c[4]) * p + c[5]) * p + c[6];
}

/* eam_alloy_fEmbed (eam_alloy.h L289-313). */
void orc_eam_embed_one(const orc_eam_tables* t, double rho, int itype, double* phi, double* fp) {
  double p = rho * t->rdrho + 1.0;
  int m = (int)p;
  if (m > t->nrho - 1) m = t->nrho - 1;
  if (m < 1) m = 1;
  p -= m;
  if (p > 1.0) p = 1.0;
  const double* c = t->frho + ((size_t)itype * (t->nrho + 1) + m) * 8;
  double f = (c[0] * p + c[1]) * p + c[2];
  double e = ((c[3] * p + c[4]) * p + c[5]) * p + c[6];
  if (rho > t->rhomax) e += f * (rho - t->rhomax);
  *phi = e * t->conv_frho;
  *fp = f * t->conv_frho;
}

/* eam_alloy_mm_force (eam_alloy.h L222-265): fpair such that the force on i
 * is dr * fpair (dr = r_j - r_i), and the pair energy phi. */
void orc_eam_pair_force(const orc_eam_tables* t, double r, double fpi, double fpj, int itype, int jtype,
                        double* fpair, double* phi_out) {
  int m;
  double p;
  r_knot(t, r, &m, &p);
  const double* ci = t->rhor + ((size_t)itype * (t->nr + 1) + m) * 8;
  const double rhoip = (ci[0] * p + ci[1]) * p + ci[2];
  const double* cj = t->rhor + ((size_t)jtype * (t->nr + 1) + m) * 8;
  const double rhojp = (cj[0] * p + cj[1]) * p + cj[2];
  const double* c = t->z2r + ((size_t)z2r_index(itype, jtype) * (t->nr + 1) + m) * 8;
  const double z2p = (c[0] * p + c[1]) * p + c[2];
  const double z2 = ((c[3] * p + c[4]) * p + c[5]) * p + c[6];
  const double recip = 1.0 / r;
  double phi = z2 * recip;
  const double phip = (z2p * recip - phi * recip) * t->conv_z2r;
  phi *= t->conv_z2r;
  const double psip = fpi * rhojp + fpj * rhoip + phip;
  *fpair = psip * recip;
  *phi_out = phi;
}

/* Density pass, SymRhoOp without Newton symmetry (eam_force_op_multimat.h
 * L123-171): rho_i = sum over list pairs with d2 <= rcut^2 of rho_{t_j}(r). */
void orc_eam_density(int64_t n, const double* x, const double* y, const double* z, const uint8_t* type,
                     const int64_t* off, const int32_t* nbr, const int8_t* img, const double L[3],
                     const orc_eam_tables* t, double rcut, double* rho) {
  const double rc2 = rcut * rcut;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    double acc = 0.0;
    for (int64_t k = off[i]; k < off[i + 1]; ++k) {
      const int nn[3] = {img[3 * k], img[3 * k + 1], img[3 * k + 2]};
      double dx, dy, dz;
      const int64_t j = nbr[k];
      const double d2 = pair_d2(x, y, z, i, j, nn, L, &dx, &dy, &dz);
      if (!(d2 <= rc2)) continue;
      acc += orc_eam_rho(t, sqrt(d2), type[j], type[i]);
    }
    rho[i] = 0.0 + acc; /* parallel_memset(0) then += at context stop */
  }
}

/* Embedding pass, Rho2EmbOp (eam_force_op_multimat.h L174-197): in place
 * rho -> F'(rho); ep += F(rho) when ep is given. */
void orc_eam_embed(int64_t n, const uint8_t* type, const orc_eam_tables* t, double* rho_dEmb, double* ep) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double phi, fp;
    orc_eam_embed_one(t, rho_dEmb[i], type[i], &phi, &fp);
    rho_dEmb[i] = fp;
    if (ep) ep[i] += phi;
  }
}

/* Force pass, SymForceOp without Newton symmetry (eam_force_op_multimat.h
 * L223-304): f_i = sum dr*fpair; with ep: ep_i += sum phi/2, vir_i += sum
 * -1/2 (dr*fpair) (x) dr.  Forces are set (zero_force_energy ran before);
 * ep is accumulated on top of the embedding energy. */
void orc_eam_force(int64_t n, const double* x, const double* y, const double* z, const uint8_t* type,
                   const int64_t* off, const int32_t* nbr, const int8_t* img, const double L[3],
                   const orc_eam_tables* t, double rcut, const double* fp, double* fx, double* fy,
                   double* fz, double* ep, double* vir) {
  const double rc2 = rcut * rcut;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    double _fx = 0., _fy = 0., _fz = 0., _ep = 0., _v[9] = {0};
    const double fpi = fp[i];
    const int ti = type[i];
    for (int64_t k = off[i]; k < off[i + 1]; ++k) {
      const int nn[3] = {img[3 * k], img[3 * k + 1], img[3 * k + 2]};
      double dx, dy, dz;
      const int64_t j = nbr[k];
      const double d2 = pair_d2(x, y, z, i, j, nn, L, &dx, &dy, &dz);
      if (!(d2 <= rc2)) continue;
      double fpair, phi;
      orc_eam_pair_force(t, sqrt(d2), fpi, fp[j], ti, type[j], &fpair, &phi);
      const double fex = dx * fpair, fey = dy * fpair, fez = dz * fpair;
      _fx += fex; _fy += fey; _fz += fez;
      _ep += .5 * phi;
      add_vir(_v, fex, fey, fez, dx, dy, dz);
    }
    fx[i] = _fx; fy[i] = _fy; fz[i] = _fz;
    if (ep) ep[i] += _ep;
    if (vir) for (int q = 0; q < 9; ++q) vir[9 * i + q] = _v[q];
  }
}

/* Force-matching + energy loss of lj_compute_force and its gradient with
 * respect to (epsilon, sigma):
 *   L = wF sum_i |F_i - F*_i|^2 + wE sum_i (E_i - E*_i)^2,
 *   F_i = sum_j g(r) d_ij with g = (de/dr)/r, d_ij = r_j - r_i,
 *   E_i = 1/2 sum_j (e(r) - e(rc)),
 * so dL/dtheta = sum_i 2wF (F_i - F*_i) . sum_j dg/dtheta d_ij
 *                + 2wE (E_i - E*_i) 1/2 sum_j (de/dtheta - de(rc)/dtheta),
 * with de/deps = e/eps, de/dsigma = 4 eps (12 s^12 - 6 s^6)/sigma, s = sigma/r
 * (lennard_jones.h L41-50).  Forces and energies are recomputed here. */
double orc_lj_loss_grad(int64_t n, const double* x, const double* y, const double* z, const int64_t* off,
                        const int32_t* nbr, const int8_t* img, const double L[3], const orc_lj_params* p,
                        const double* fxt, const double* fyt, const double* fzt, const double* et, double wF,
                        double wE, double grad[2]) {
  const double eps = p->epsilon, sig = p->sigma, rc2 = p->rcut * p->rcut;
  const double ecut = orc_lj_energy_cut(eps, sig, p->rcut);
  const double sc = sig / p->rcut, sc6 = sc * sc * sc * sc * sc * sc, sc12 = sc6 * sc6;
  const double decut_deps = ecut / eps, decut_dsig = 4. * eps * (12. * sc12 - 6. * sc6) / sig;
  double loss = 0., ge = 0., gs = 0.;
#pragma omp parallel for schedule(static) reduction(+ : loss, ge, gs)
  for (int64_t i = 0; i < n; ++i) {
    double F[3] = {0., 0., 0.}, E = 0.;
    for (int64_t k = off[i]; k < off[i + 1]; ++k) {
      const int nn[3] = {img[3 * k], img[3 * k + 1], img[3 * k + 2]};
      double dx, dy, dz;
      const double d2 = pair_d2(x, y, z, i, nbr[k], nn, L, &dx, &dy, &dz);
      if (!(d2 <= rc2)) continue;
      const double r = sqrt(d2);
      double e, de;
      orc_lj_pair(eps, sig, r, &e, &de);
      const double g = de / r;
      F[0] += g * dx; F[1] += g * dy; F[2] += g * dz;
      E += .5 * (e - ecut);
    }
    const double dF[3] = {F[0] - fxt[i], F[1] - fyt[i], F[2] - fzt[i]};
    const double dE = E - et[i];
    loss += wF * (dF[0] * dF[0] + dF[1] * dF[1] + dF[2] * dF[2]) + wE * dE * dE;
    double gi_e = 0., gi_s = 0.;
    for (int64_t k = off[i]; k < off[i + 1]; ++k) {
      const int nn[3] = {img[3 * k], img[3 * k + 1], img[3 * k + 2]};
      double dx, dy, dz;
      const double d2 = pair_d2(x, y, z, i, nbr[k], nn, L, &dx, &dy, &dz);
      if (!(d2 <= rc2)) continue;
      const double r = sqrt(d2);
      const double s = sig / r, s2 = s * s, s6 = s2 * s2 * s2, s12 = s6 * s6;
      const double e = 4. * eps * (s12 - s6);
      const double g = -24. * eps * (2. * s12 - s6) / d2;             /* (de/dr)/r */
      const double dg_deps = g / eps;
      const double dg_dsig = -24. * eps * (24. * s12 - 6. * s6) / (d2 * sig);
      const double proj = dF[0] * dx + dF[1] * dy + dF[2] * dz;
      gi_e += 2. * wF * proj * dg_deps + wE * dE * (e / eps - decut_deps);
      gi_s += 2. * wF * proj * dg_dsig + wE * dE * (4. * eps * (12. * s12 - 6. * s6) / sig - decut_dsig);
    }
    ge += gi_e;
    gs += gi_s;
  }
  grad[0] = ge;
  grad[1] = gs;
  return loss;
}

/* ------------------------------------------------------------------------ */
/* johnson_force: analytic single-element EAM                               */
/* ------------------------------------------------------------------------ */

/* One c1/(1 + (x-c)^20) term and its r-derivative (johnson.h L55-94). */
static void ej_term(double pre, double k, double x, double c, double ire, double* v, double* dv) {
  const double c1 = pre * exp(-k * (x - 1.));
  const double c2 = x - c;
  const double c3 = pow(c2, 20.);
  const double den = 1. + c3;
  const double dnum = -k * c1;
  const double dden = 20. * c3 / c2;
  *v += c1 / den;
  *dv += ire * (dnum * den - c1 * dden) / (den * den);
}

/* eam_johnson_phi (johnson.h L55-94) */
void orc_ej_phi(const orc_johnson_params* p, double r, double* phi, double* dphi) {
  const double x = r / p->re, ire = 1. / p->re;
  *phi = 0.;
  *dphi = 0.;
  ej_term(p->A, p->alpha, x, p->kappa, ire, phi, dphi);
  ej_term(-p->B, p->beta, x, p->lambda, ire, phi, dphi);
}

/* eam_johnson_rho (johnson.h L101-118) */
void orc_ej_rho(const orc_johnson_params* p, double r, double* rho, double* drho) {
  const double x = r / p->re, ire = 1. / p->re;
  *rho = 0.;
  *drho = 0.;
  ej_term(p->fe, p->beta, x, p->lambda, ire, rho, drho);
}

/* eam_johnson_fEmbed (johnson.h L125-176): three branches split at
 * 0.85 rhoe and 1.15 rhoe. */
void orc_ej_embed(const orc_johnson_params* p, double rho, double* f, double* df) {
  const double rhon = 0.85 * p->rhoe, rho0 = 1.15 * p->rhoe;
  if (rho < rhon) {
    const double t = rho / rhon - 1.;
    *f = p->Fn0 + p->Fn1 * t + p->Fn2 * (t * t) + p->Fn3 * (t * (t * t));
    *df = (p->Fn1 + 2. * p->Fn2 * t + 3. * p->Fn3 * (t * t)) * (1. / rhon);
  } else if (rho < rho0) {
    const double t = rho * (1. / p->rhoe) - 1.;
    *f = p->F0 + p->F1 * t + p->F2 * (t * t) + p->F3 * (t * (t * t));
    *df = (p->F1 + 2. * p->F2 * t + 3. * p->F3 * (t * t)) * (1. / p->rhoe);
  } else {
    const double s = rho * (1. / p->rhoe);
    const double se = pow(s, p->eta);
    const double lse = log(se);
    *f = p->Fo * (1. - lse) * se;
    *df = (-p->eta * se + (1. - lse) * p->eta * se) * (p->Fo * (1. / p->rhoe) / s);
  }
}

/* sutton_chen_force: phi = epsilon (a0/r)^n (sutton_chen.h L40-46), rho =
 * (a0/r)^m (L48-56), F = -c epsilon sqrt(rho) (L58-66), derivatives as there */
void orc_sc_phi(const orc_sutton_chen_params* p, double r, double* phi, double* dphi) {
  const double ratio = p->a0 / r;
  *phi = p->epsilon * pow(ratio, p->n);
  *dphi = -1 * p->n * *phi / r;
}

void orc_sc_rho(const orc_sutton_chen_params* p, double r, double* rho, double* drho) {
  const double ratio = p->a0 / r;
  *rho = pow(ratio, p->m);
  *drho = -1 * p->m * *rho / r;
}

void orc_sc_embed(const orc_sutton_chen_params* p, double rho, double* f, double* df) {
  const double sq = sqrt(rho);
  *f = -1. * p->c * p->epsilon * sq;
  *df = 0.5 * *f / (rho > 0 ? rho : 0);
}

typedef void (*orc_pair_fn)(const void* p, double r, double* v, double* dv);

/* The two passes of the mono-material template (eam_potential.cu L125-170):
 * EmbOp (eam_force_op_singlemat.h L39-84): rho_i, ep_i = F(rho_i), F'_i;
 * ForceOp (L86-171): de = (rho'(F'_i + F'_j) + phi')/r, f_i += de*dr,
 * ep_i += phi/2, vir_i += -1/2 f (x) dr.  fp receives F'. */
static void analytic_two_pass(int64_t n, const double* x, const double* y, const double* z, const int64_t* off,
                              const int32_t* nbr, const int8_t* img, const double L[3], const void* p,
                              orc_pair_fn rho_fn, orc_pair_fn phi_fn, orc_pair_fn emb_fn, double rcut,
                              double* fp, double* fx, double* fy, double* fz, double* ep, double* vir) {
  const double rc2 = rcut * rcut;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    double rho = 0.;
    for (int64_t k = off[i]; k < off[i + 1]; ++k) {
      const int nn[3] = {img[3 * k], img[3 * k + 1], img[3 * k + 2]};
      double dx, dy, dz;
      const double d2 = pair_d2(x, y, z, i, nbr[k], nn, L, &dx, &dy, &dz);
      if (!(d2 <= rc2)) continue;
      double v, dv;
      rho_fn(p, sqrt(d2), &v, &dv);
      rho += v;
    }
    double f, df;
    emb_fn(p, rho, &f, &df);
    fp[i] = df;
    if (ep) ep[i] = f;
  }
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    double _fx = 0., _fy = 0., _fz = 0., _ep = 0., _v[9] = {0};
    for (int64_t k = off[i]; k < off[i + 1]; ++k) {
      const int nn[3] = {img[3 * k], img[3 * k + 1], img[3 * k + 2]};
      double dx, dy, dz;
      const int64_t j = nbr[k];
      const double d2 = pair_d2(x, y, z, i, j, nn, L, &dx, &dy, &dz);
      if (!(d2 <= rc2)) continue;
      const double r = sqrt(d2);
      double rh, drh, ph, dph;
      rho_fn(p, r, &rh, &drh);
      phi_fn(p, r, &ph, &dph);
      const double de = (drh * (fp[i] + fp[j]) + dph) / r;
      const double fex = de * dx, fey = de * dy, fez = de * dz;
      _fx += fex; _fy += fey; _fz += fez;
      _ep += .5 * ph;
      add_vir(_v, fex, fey, fez, dx, dy, dz);
    }
    fx[i] = _fx; fy[i] = _fy; fz[i] = _fz;
    if (ep) ep[i] += _ep;
    if (vir) for (int q = 0; q < 9; ++q) vir[9 * i + q] = _v[q];
  }
}

static void ej_rho_v(const void* p, double r, double* v, double* dv) { orc_ej_rho((const orc_johnson_params*)p, r, v, dv); }
static void ej_phi_v(const void* p, double r, double* v, double* dv) { orc_ej_phi((const orc_johnson_params*)p, r, v, dv); }
static void ej_emb_v(const void* p, double r, double* v, double* dv) { orc_ej_embed((const orc_johnson_params*)p, r, v, dv); }
static void sc_rho_v(const void* p, double r, double* v, double* dv) { orc_sc_rho((const orc_sutton_chen_params*)p, r, v, dv); }
static void sc_phi_v(const void* p, double r, double* v, double* dv) { orc_sc_phi((const orc_sutton_chen_params*)p, r, v, dv); }
static void sc_emb_v(const void* p, double r, double* v, double* dv) { orc_sc_embed((const orc_sutton_chen_params*)p, r, v, dv); }

void orc_ej_forces(int64_t n, const double* x, const double* y, const double* z, const int64_t* off,
                   const int32_t* nbr, const int8_t* img, const double L[3], const orc_johnson_params* p,
                   double rcut, double* fp, double* fx, double* fy, double* fz, double* ep, double* vir) {
  analytic_two_pass(n, x, y, z, off, nbr, img, L, p, ej_rho_v, ej_phi_v, ej_emb_v, rcut, fp, fx, fy, fz, ep, vir);
}

void orc_sc_forces(int64_t n, const double* x, const double* y, const double* z, const int64_t* off,
                   const int32_t* nbr, const int8_t* img, const double L[3], const orc_sutton_chen_params* p,
                   double rcut, double* fp, double* fx, double* fy, double* fz, double* ep, double* vir) {
  analytic_two_pass(n, x, y, z, off, nbr, img, L, p, sc_rho_v, sc_phi_v, sc_emb_v, rcut, fp, fx, fy, fz, ep, vir);
}

/* ------------------------------------------------------------------------ */
/* Integration, accel, thermo                                               */
/* ------------------------------------------------------------------------ */

/* push_f_v_r: r += v*dt' + a*dt'^2/2, dt' = dt*dt_scale (identity xform;
 * formula restated in push_vec3_2nd_order_xform_minimization.cpp L33-38). */
void orc_push_f_v_r(int64_t n, double* x, double* y, double* z, const double* vx, const double* vy,
                    const double* vz, const double* ax, const double* ay, const double* az, double dt,
                    double dt_scale) {
  const double h = dt * dt_scale;
  const double h2 = h * h * 0.5;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    x[i] += vx[i] * h + ax[i] * h2;
    y[i] += vy[i] * h + ay[i] * h2;
    z[i] += vz[i] * h + az[i] * h2;
  }
}

/* push_f_v: v += a*dt*dt_scale. */
void orc_push_f_v(int64_t n, double* vx, double* vy, double* vz, const double* ax, const double* ay,
                  const double* az, double dt, double dt_scale) {
  const double h = dt * dt_scale;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    vx[i] += ax[i] * h;
    vy[i] += ay[i] * h;
    vz[i] += az[i] * h;
  }
}

/* push_f_v_r_xform_minimization, identity-xform branch
 * (push_vec3_2nd_order_xform_minimization.cpp L116-149): r += a*dt'^2/2.
 * tolF > 0 additionally clips each acceleration component to [-tolF, tolF]
 * and writes the clipped value back (the clipping of the same file's
 * non-identity branch, L174-205); tolF <= 0 is the identity branch as is. */
void orc_push_min(int64_t n, double* x, double* y, double* z, double* ax, double* ay, double* az,
                  const uint8_t* type, const double* masses, double dt, double dt_scale, double tolF) {
  (void)type;
  (void)masses;
  const double h = dt * dt_scale;
  const double h2 = h * h * 0.5;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    if (tolF > 0.0) {
      if (fabs(ax[i]) > tolF) ax[i] = ax[i] > 0. ? tolF : -tolF;
      if (fabs(ay[i]) > tolF) ay[i] = ay[i] > 0. ? tolF : -tolF;
      if (fabs(az[i]) > tolF) az[i] = az[i] > 0. ? tolF : -tolF;
    }
    x[i] += ax[i] * h2;
    y[i] += ay[i] * h2;
    z[i] += az[i] * h2;
  }
}

/* force_to_accel (force_to_accel.cu L42-48): a = f / m[type], in place. */
void orc_force_to_accel(int64_t n, double* fx, double* fy, double* fz, const uint8_t* type,
                        const double* masses) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const double m = masses[type ? type[i] : 0];
    fx[i] /= m;
    fy[i] /= m;
    fz[i] /= m;
  }
}

/* simulation_thermodynamic_state (L101-163): the 27 reduced doubles, in the
 * reference's order: virial(9), ke_tensor(9) = 1/2 sum m v(x)v, momentum(3),
 * kinetic energy vector(3) = 1/2 sum m v*v, potential energy, mass, count.
 * Summed in fixed 4096-atom chunks so the result is thread-count independent. */
void orc_thermo(int64_t n, const double* vx, const double* vy, const double* vz, const double* ep,
                const double* vir, const uint8_t* type, const double* masses, double out[27]) {
  const int64_t CH = 4096;
  const int64_t nch = (n + CH - 1) / CH;
  double* part = (double*)calloc((size_t)(nch > 0 ? nch : 1) * 26, sizeof(double));
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nch; ++c) {
    double* s = part + 26 * c;
    const int64_t e = (c + 1) * CH < n ? (c + 1) * CH : n;
    for (int64_t i = c * CH; i < e; ++i) {
      const double m = masses[type ? type[i] : 0];
      const double v[3] = {vx[i], vy[i], vz[i]};
      if (vir) for (int q = 0; q < 9; ++q) s[q] += vir[9 * i + q];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) s[9 + 3 * a + b] += v[a] * v[b] * m;
      for (int a = 0; a < 3; ++a) s[18 + a] += v[a] * m;
      for (int a = 0; a < 3; ++a) s[21 + a] += v[a] * v[a] * m;
      if (ep) s[24] += ep[i];
      s[25] += m;
    }
  }
  for (int q = 0; q < 27; ++q) out[q] = 0.0;
  for (int64_t c = 0; c < nch; ++c)
    for (int q = 0; q < 26; ++q) out[q] += part[26 * c + q];
  for (int q = 9; q < 18; ++q) out[q] *= 0.5;
  for (int q = 21; q < 24; ++q) out[q] *= 0.5;
  out[26] = (double)n;
  free(part);
}

/* ------------------------------------------------------------------------ */
/* Parameter adjoint of the force-matching + energy loss (single element)    */
/* ------------------------------------------------------------------------ */

static inline double sp_val(const double* c, double p) { return ((c[3] * p + c[4]) * p + c[5]) * p + c[6]; }
static inline double sp_der(const double* c, double p) { return (c[0] * p + c[1]) * p + c[2]; }

static inline void rho_knot(const orc_eam_tables* t, double rho, int* m, double* p) {
  double pp = rho * t->rdrho + 1.0;
  int mm = (int)pp;
  if (mm > t->nrho - 1) mm = t->nrho - 1;
  if (mm < 1) mm = 1;
  pp -= mm;
  if (pp > 1.0) pp = 1.0;
  *m = mm;
  *p = pp;
}

/* Forward in the reference's formulas (eam_alloy.h L198-313 with conv = 1),
 * then the reverse sweep:
 *   s_ij = gF_i . u_ij                     (dL/dpsi'_ij, psi' = F'_i rho'_ij + F'_j rho'_ij + phi'_ij)
 *   G_i  = sum_j (s_ij + s_ji) rho'_ij     (dL/dF'_i through the forces)
 *   lam_i = gE_i F'_i + G_i F''_i          (dL/drho_i)
 * and every spline evaluation is differentiated with respect to the
 * parameters by evaluating the same formula on the derivative splines. */
double orc_eam_loss_grad(int64_t n, const double* x, const double* y, const double* z, const int64_t* off,
                         const int32_t* nbr, const int8_t* img, const double L[3], const orc_eam_tables* t,
                         double rcut, const orc_eam_dtables* d, const double* Ft, const double* Et, double wF,
                         double wE, double* grad, double* F, double* E) {
  const double rc2 = rcut * rcut;
  const int np = d->nparam;
  const size_t kr = (size_t)t->nr + 1, kp = (size_t)t->nrho + 1;
  double* rho = (double*)calloc((size_t)n + 1, sizeof(double));
  double* fp = (double*)calloc((size_t)n + 1, sizeof(double));
  double* fpp = (double*)calloc((size_t)n + 1, sizeof(double));
  double* f = (double*)calloc(3 * (size_t)n + 1, sizeof(double));
  double* e = (double*)calloc((size_t)n + 1, sizeof(double));
  double* gF = (double*)calloc(3 * (size_t)n + 1, sizeof(double));
  double* gE = (double*)calloc((size_t)n + 1, sizeof(double));
  double* G = (double*)calloc((size_t)n + 1, sizeof(double));
  double* gacc = (double*)calloc((size_t)np + 1, sizeof(double));
#define PAIR_BEGIN                                                               \
  for (int64_t k = off[i]; k < off[i + 1]; ++k) {                                \
    const int nn[3] = {img[3 * k], img[3 * k + 1], img[3 * k + 2]};              \
    double dx, dy, dz;                                                           \
    const int64_t j = nbr[k];                                                    \
    const double d2 = pair_d2(x, y, z, i, j, nn, L, &dx, &dy, &dz);              \
    if (!(d2 <= rc2)) continue;                                                  \
    const double r = sqrt(d2);                                                   \
    int m;                                                                       \
    double p;                                                                    \
    r_knot(t, r, &m, &p);
#define PAIR_END }
  /* forward: density, embedding */
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; ++i) {
    double acc = 0.0;
    PAIR_BEGIN
    acc += sp_val(t->rhor + (size_t)m * 8, p);
    PAIR_END
    rho[i] = acc;
    int mq;
    double q;
    rho_knot(t, acc, &mq, &q);
    const double* c = t->frho + (size_t)mq * 8;
    double fv = sp_der(c, q), ev = sp_val(c, q);
    double f2 = (2.0 * c[0] * q + c[1]) * t->rdrho;
    if (acc > t->rhomax) {
      ev += fv * (acc - t->rhomax);
      f2 = 0.0;
    }
    fp[i] = fv;
    fpp[i] = f2;
    e[i] = ev;
  }
  /* forward: forces and pair energies */
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; ++i) {
    double sx = 0., sy = 0., sz = 0., se = 0.;
    PAIR_BEGIN
    const double* cr = t->rhor + (size_t)m * 8;
    const double* cz = t->z2r + (size_t)m * 8;
    const double rhop = sp_der(cr, p);
    const double z2p = sp_der(cz, p), z2 = sp_val(cz, p);
    const double phi = z2 / r;
    const double phip = z2p / r - phi / r;
    const double psip = (fp[i] + fp[j]) * rhop + phip;
    sx += dx * psip / r;
    sy += dy * psip / r;
    sz += dz * psip / r;
    se += 0.5 * phi;
    PAIR_END
    f[3 * i] = sx;
    f[3 * i + 1] = sy;
    f[3 * i + 2] = sz;
    e[i] += se;
  }
  /* loss and its gradient with respect to the per-atom outputs */
  double loss = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    for (int a = 0; a < 3; ++a) {
      const double df = f[3 * i + a] - Ft[3 * i + a];
      loss += wF * df * df;
      gF[3 * i + a] = 2.0 * wF * df;
    }
    const double de = e[i] - Et[i];
    loss += wE * de * de;
    gE[i] = 2.0 * wE * de;
  }
  /* reverse sweep 1: pair terms through phi, phi' and rho'; G_i */
#pragma omp parallel
  {
    double* gl = (double*)calloc((size_t)np + 1, sizeof(double));
#pragma omp for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
      double gi = 0.0;
      PAIR_BEGIN
      const double ux = dx / r, uy = dy / r, uz = dz / r;
      const double sij = gF[3 * i] * ux + gF[3 * i + 1] * uy + gF[3 * i + 2] * uz;
      const double sji = -(gF[3 * j] * ux + gF[3 * j + 1] * uy + gF[3 * j + 2] * uz);
      const double rhop = sp_der(t->rhor + (size_t)m * 8, p);
      gi += (sij + sji) * rhop;
      const double wv = 0.5 * gE[i] / r - sij / (r * r); /* weight of dz2 */
      const double wd = sij / r;                         /* weight of dz2' */
      const double wr = sij * (fp[i] + fp[j]);            /* weight of drho' */
      for (int q = 0; q < np; ++q) {
        const double* dz2 = d->dz2r + ((size_t)q * kr + m) * 8;
        const double* drh = d->drhor + ((size_t)q * kr + m) * 8;
        gl[q] += wv * sp_val(dz2, p) + wd * sp_der(dz2, p) + wr * sp_der(drh, p);
      }
      PAIR_END
      G[i] = gi;
    }
#pragma omp critical
    for (int q = 0; q < np; ++q) gacc[q] += gl[q];
    free(gl);
  }
  /* reverse sweep 2: embedding terms and rho values through lam_i */
#pragma omp parallel
  {
    double* gl = (double*)calloc((size_t)np + 1, sizeof(double));
#pragma omp for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
      const double lam = gE[i] * fp[i] + G[i] * fpp[i];
      int mq;
      double q;
      rho_knot(t, rho[i], &mq, &q);
      const double over = rho[i] > t->rhomax ? rho[i] - t->rhomax : 0.0;
      for (int a = 0; a < np; ++a) {
        const double* c = d->dfrho + ((size_t)a * kp + mq) * 8;
        const double dfp = sp_der(c, q);
        gl[a] += gE[i] * (sp_val(c, q) + dfp * over) + G[i] * dfp;
      }
      PAIR_BEGIN
      for (int a = 0; a < np; ++a) gl[a] += lam * sp_val(d->drhor + ((size_t)a * kr + m) * 8, p);
      PAIR_END
    }
#pragma omp critical
    for (int a = 0; a < np; ++a) gacc[a] += gl[a];
    free(gl);
  }
#undef PAIR_BEGIN
#undef PAIR_END
  for (int q = 0; q < np; ++q) grad[q] += gacc[q];
  if (F) memcpy(F, f, sizeof(double) * 3 * (size_t)n);
  if (E) memcpy(E, e, sizeof(double) * (size_t)n);
  free(rho); free(fp); free(fpp); free(f); free(e); free(gF); free(gE); free(G); free(gacc);
  return loss;
}

/* ------------------------------------------------------------------------ */
/* verlet_nve driver (config_numerical_schemes.msp L23-52)                   */
/* ------------------------------------------------------------------------ */

typedef struct {
  int64_t* off;
  int32_t* nbr;
  int8_t* img;
  int64_t cap;
} orc_list;

static int list_rebuild(orc_list* l, int64_t n, double* x, double* y, double* z, const uint64_t* id,
                        const double lo[3], const double hi[3], double R) {
  if (orc_wrap(n, x, y, z, lo, hi) != 0) return -3;
  int64_t tot = orc_build_neighbors(n, x, y, z, id, lo, hi, R, l->off, l->cap, l->nbr, l->img);
  if (tot < 0) return -1;
  if (tot > l->cap) {
    free(l->nbr);
    free(l->img);
    l->cap = tot + tot / 8 + 64;
    l->nbr = (int32_t*)malloc(sizeof(int32_t) * (size_t)l->cap);
    l->img = (int8_t*)malloc(3 * (size_t)l->cap);
    tot = orc_build_neighbors(n, x, y, z, id, lo, hi, R, l->off, l->cap, l->nbr, l->img);
  }
  return 0;
}

static void compute_pair_forces(int64_t n, const double* x, const double* y, const double* z,
                                const uint8_t* type, const orc_list* l, const double L[3], int pot_kind,
                                const void* pot, double* fx, double* fy, double* fz, double* ep, double* vir) {
  if (pot_kind == ORC_POT_LJ)
    orc_lj_force(n, x, y, z, l->off, l->nbr, l->img, L, (const orc_lj_params*)pot, fx, fy, fz, ep, vir);
  else
    orc_lj_multi_force(n, x, y, z, type, l->off, l->nbr, l->img, L, (const orc_lj_multi_params*)pot, fx,
                       fy, fz, ep, vir);
}

/* list builds of the last orc_run_nve / orc_run_minimize call */
static int64_t g_list_builds = 0;

int64_t orc_last_list_builds(void) { return g_list_builds; }

/* particle_displ_over (config_move_particles.msp L19-22, L116-118): 1 when
 * some atom moved more than skin/2 since rref was taken; |dr|^2 summed x, y,
 * z in that order (the file is compiled without contraction). */
static int displ_over(int64_t n, const double* x, const double* y, const double* z, const double* rref,
                      double skin) {
  const double thr = 0.5 * skin, thr2 = thr * thr;
  int over = 0;
#pragma omp parallel for schedule(static) reduction(| : over)
  for (int64_t i = 0; i < n; ++i) {
    const double dx = x[i] - rref[i], dy = y[i] - rref[n + i], dz = z[i] - rref[2 * n + i];
    if (dx * dx + dy * dy + dz * dz > thr2) over = 1;
  }
  return over;
}

static void take_rref(int64_t n, const double* x, const double* y, const double* z, double* rref) {
  memcpy(rref, x, sizeof(double) * (size_t)n);
  memcpy(rref + n, y, sizeof(double) * (size_t)n);
  memcpy(rref + 2 * n, z, sizeof(double) * (size_t)n);
}

/* the list update of one step: every `every` steps, or on the displacement
 * trigger when every == -1 */
static int maybe_rebuild(orc_list* l, int64_t n, double* x, double* y, double* z, const uint64_t* id,
                         const double lo[3], const double hi[3], double R, double skin, int every, int s,
                         double* rref) {
  int rc = 0;
  if (every > 0 && s % every == 0) {
    rc = list_rebuild(l, n, x, y, z, id, lo, hi, R);
    ++g_list_builds;
  } else if (every == -1 && displ_over(n, x, y, z, rref, skin)) {
    rc = list_rebuild(l, n, x, y, z, id, lo, hi, R);
    take_rref(n, x, y, z, rref);
    ++g_list_builds;
  }
  return rc;
}

static double pot_rcut(int pot_kind, const void* pot) {
  if (pot_kind == ORC_POT_LJ) return ((const orc_lj_params*)pot)->rcut;
  if (pot_kind == ORC_POT_LJ_MULTI) return ((const orc_lj_multi_params*)pot)->rcut_max;
  if (pot_kind == ORC_POT_EAM_JOHNSON) return ((const orc_johnson_pot*)pot)->rcut;
  if (pot_kind == ORC_POT_EAM_SUTTON_CHEN) return ((const orc_sutton_chen_pot*)pot)->rcut;
  return ((const orc_eam_pot*)pot)->rcut;
}

/* Forces of the bound potential turned into accelerations: the compute_force
 * node of the step graph (eam_alloy = density, embedding, force passes). */
static void all_forces(int64_t n, const double* x, const double* y, const double* z, const uint8_t* type,
                       const orc_list* l, const double L[3], int pot_kind, const void* pot, const double* masses,
                       double* rho, double* ax, double* ay, double* az, double* ep, double* vir) {
  if (pot_kind == ORC_POT_EAM_JOHNSON) {
    const orc_johnson_pot* p = (const orc_johnson_pot*)pot;
    orc_ej_forces(n, x, y, z, l->off, l->nbr, l->img, L, &p->p, p->rcut, rho, ax, ay, az, ep, vir);
  } else if (pot_kind == ORC_POT_EAM_SUTTON_CHEN) {
    const orc_sutton_chen_pot* p = (const orc_sutton_chen_pot*)pot;
    orc_sc_forces(n, x, y, z, l->off, l->nbr, l->img, L, &p->p, p->rcut, rho, ax, ay, az, ep, vir);
  } else if (pot_kind == ORC_POT_EAM) {
    const orc_eam_pot* p = (const orc_eam_pot*)pot;
    orc_eam_density(n, x, y, z, type, l->off, l->nbr, l->img, L, &p->t, p->rcut, rho);
    for (int64_t i = 0; i < n; ++i) ep[i] = 0.0;
    orc_eam_embed(n, type, &p->t, rho, ep);
    orc_eam_force(n, x, y, z, type, l->off, l->nbr, l->img, L, &p->t, p->rcut, rho, ax, ay, az, ep, vir);
  } else {
    compute_pair_forces(n, x, y, z, type, l, L, pot_kind, pot, ax, ay, az, ep, vir);
  }
  orc_force_to_accel(n, ax, ay, az, type, masses);
}

static int run_nve_impl(int64_t n, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                        double* ax, double* ay, double* az, double* ep, const uint8_t* type, const uint64_t* id,
                        const double* masses, const double lo[3], const double hi[3], int pot_kind,
                        const void* pot, double skin, double dt, int nsteps, int rebuild_every,
                        double* thermo_out, int initial_forces) {
  const double L[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  const double R = pot_rcut(pot_kind, pot) + skin;
  orc_list l = {(int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 1)), NULL, NULL, 0};
  double* rho = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  /* per-atom virial, summed by the thermo reduction (mechanics grid flavor) */
  double* vir = thermo_out ? (double*)calloc(9 * (size_t)(n > 0 ? n : 1), sizeof(double)) : NULL;
  double* rref = (double*)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
  int rc = 0;
  g_list_builds = 1;
  if ((rc = list_rebuild(&l, n, x, y, z, id, lo, hi, R)) != 0) goto done;
  take_rref(n, x, y, z, rref);
  if (initial_forces) {
    all_forces(n, x, y, z, type, &l, L, pot_kind, pot, masses, rho, ax, ay, az, ep, vir);
  } else {
    for (int64_t i = 0; i < n; ++i) ep[i] = 0.0;
  }
  if (thermo_out) orc_thermo(n, vx, vy, vz, ep, vir, type, masses, thermo_out);
  for (int s = 1; s <= nsteps; ++s) {
    orc_push_f_v_r(n, x, y, z, vx, vy, vz, ax, ay, az, dt, 1.0);
    orc_push_f_v(n, vx, vy, vz, ax, ay, az, dt, 0.5);
    if ((rc = maybe_rebuild(&l, n, x, y, z, id, lo, hi, R, skin, rebuild_every, s, rref)) != 0) goto done;
    all_forces(n, x, y, z, type, &l, L, pot_kind, pot, masses, rho, ax, ay, az, ep, vir);
    orc_push_f_v(n, vx, vy, vz, ax, ay, az, dt, 0.5);
    if (thermo_out) orc_thermo(n, vx, vy, vz, ep, vir, type, masses, thermo_out + 27 * s);
  }
done:
  free(l.off);
  free(l.nbr);
  free(l.img);
  free(rho);
  free(vir);
  free(rref);
  return rc;
}

int orc_run_nve(int64_t n, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                double* ax, double* ay, double* az, double* ep, const uint8_t* type, const uint64_t* id,
                const double* masses, const double lo[3], const double hi[3], int pot_kind,
                const void* pot, double skin, double dt, int nsteps, int rebuild_every,
                double* thermo_out) {
  return run_nve_impl(n, x, y, z, vx, vy, vz, ax, ay, az, ep, type, id, masses, lo, hi, pot_kind, pot, skin, dt,
                      nsteps, rebuild_every, thermo_out, 1);
}

int orc_run_nve_from(int64_t n, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                     double* ax, double* ay, double* az, double* ep, const uint8_t* type, const uint64_t* id,
                     const double* masses, const double lo[3], const double hi[3], int pot_kind,
                     const void* pot, double skin, double dt, int nsteps, int rebuild_every,
                     double* thermo_out) {
  return run_nve_impl(n, x, y, z, vx, vy, vz, ax, ay, az, ep, type, id, masses, lo, hi, pot_kind, pot, skin, dt,
                      nsteps, rebuild_every, thermo_out, 0);
}

int orc_run_minimize(int64_t n, double* x, double* y, double* z, double* ax, double* ay, double* az,
                     double* ep, const uint8_t* type, const uint64_t* id, const double* masses,
                     const double lo[3], const double hi[3], int pot_kind, const void* pot, double skin,
                     double dt, double tolF, int nsteps, int rebuild_every) {
  const double L[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  const double R = pot_rcut(pot_kind, pot) + skin;
  orc_list l = {(int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 1)), NULL, NULL, 0};
  double* rho = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  double* rref = (double*)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
  int rc = 0;
  g_list_builds = 1;
  if ((rc = list_rebuild(&l, n, x, y, z, id, lo, hi, R)) != 0) goto done;
  take_rref(n, x, y, z, rref);
  for (int s = 1; s <= nsteps; ++s) {
    all_forces(n, x, y, z, type, &l, L, pot_kind, pot, masses, rho, ax, ay, az, ep, NULL);
    orc_push_min(n, x, y, z, ax, ay, az, type, masses, dt, 1.0, tolF);
    if ((rc = maybe_rebuild(&l, n, x, y, z, id, lo, hi, R, skin, rebuild_every, s, rref)) != 0) goto done;
  }
done:
  free(l.off);
  free(l.nbr);
  free(l.img);
  free(rho);
  free(rref);
  return rc;
}
