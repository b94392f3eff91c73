/*
 * gbmd_oracle.h -- CPU FP64 restatement of exaStamp's per-timestep MD hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle (and the
 * timed CPU baseline) for the GB300 kernels in exastamp_gb300/csrc.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm
 * may load it.  Nothing in the product path calls it.
 *
 * Parity status: the per-pair arithmetic below restates the reference's own
 * in-tree functions (cited per function).  The traversal contracts it also
 * restates (cell binning, the neighbour pair set, the Verlet push) live in
 * exaNBody v2.0.1, which is not part of the reference tree; for those the
 * oracle follows the contracts visible at the reference's call sites and is
 * cross-checked against an O(N^2) all-image direct sum in tests.
 *
 * Conventions (shared bit-for-bit with the GPU path):
 *   - arrays are SoA, FP64, in the caller's atom order;
 *   - the box is orthorhombic and periodic in x, y and z, [lo, hi);
 *   - an image shift n (int8 x3, n in {-1,0,1}) means the neighbour's position
 *     is x_j + n*L, and dr = (x_j + n*L) - x_i, d2 = dx*dx + dy*dy + dz*dz
 *     evaluated left to right with no FMA contraction.
 */
#ifndef GBMD_ORACLE_H
#define GBMD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Tabulated eam_alloy potential: flattened 7-coefficient splines, 8 doubles
 * per knot (the 8th is padding), knots 0..n per table (knot 0 unused).
 * Layout follows eam_alloy.cpp L251-273 of the reference. */
typedef struct {
  int nelements, nr, nrho, pad_;
  double rdr, rdrho, rhomax, conv_z2r, conv_frho;
  const double* frho; /* nelements           x (nrho+1) x 8 */
  const double* rhor; /* nelements           x (nr+1)   x 8 */
  const double* z2r;  /* nel*(nel+1)/2       x (nr+1)   x 8 */
} orc_eam_tables;

/* eam_alloy operator parameters: the tables plus the operator's rcut slot
 * (eam_potential_multimat.cu L91), which is the traversal cutoff. */
typedef struct {
  orc_eam_tables t;
  double rcut;
} orc_eam_pot;

/* Kinds for orc_run_nve */
enum { ORC_POT_LJ = 0, ORC_POT_LJ_MULTI = 1, ORC_POT_EAM = 2, ORC_POT_EAM_JOHNSON = 3, ORC_POT_EAM_SUTTON_CHEN = 4 };

/* johnson_force parameters, EamJohnsonParameters order (johnson.h L28-49) */
typedef struct {
  double re, fe, rhoe, alpha, beta, A, B, kappa, lambda, Fn0, Fn1, Fn2, Fn3, F0, F1, F2, F3, Fo, eta;
} orc_johnson_params;

typedef struct {
  orc_johnson_params p;
  double rcut;
} orc_johnson_pot;

/* sutton_chen_force parameters, EamSuttonChenParameters order (sutton_chen.h L30-37) */
typedef struct {
  double c, epsilon, a0, n, m;
} orc_sutton_chen_params;

typedef struct {
  orc_sutton_chen_params p;
  double rcut;
} orc_sutton_chen_pot;

typedef struct {
  double epsilon, sigma, rcut;
} orc_lj_params;

typedef struct {
  int ntypes, pad_;
  const double* epsilon; /* ntypes x ntypes, symmetric */
  const double* sigma;   /* ntypes x ntypes, symmetric */
  const double* rcut;    /* ntypes x ntypes, symmetric */
  double rcut_max;
} orc_lj_multi_params;

int orc_grid_dims(const double lo[3], const double hi[3], double R, int nc[3]);
int64_t orc_wrap(int64_t n, double* x, double* y, double* z, const double lo[3], const double hi[3]);
int64_t orc_build_neighbors(int64_t n, const double* x, const double* y, const double* z,
                            const uint64_t* id, const double lo[3], const double hi[3], double R,
                            int64_t* offsets, int64_t cap, int32_t* nbr, int8_t* img);
int64_t orc_build_neighbors_first(int64_t n, int64_t nlist, const double* x, const double* y, const double* z,
                                  const uint64_t* id, const double lo[3], const double hi[3], double R,
                                  int64_t* offsets, int64_t cap, int32_t* nbr, int8_t* img);
int64_t orc_brute_pairs(int64_t n, const double* x, const double* y, const double* z,
                        const double lo[3], const double hi[3], double R, int64_t cap,
                        int32_t* pi, int32_t* pj, int8_t* img);

double orc_lj_energy_cut(double epsilon, double sigma, double rcut);
void orc_lj_pair(double epsilon, double sigma, double r, double* e, double* de);
void orc_lj_atom_buffer(double epsilon, double sigma, double ecut, int n, const double* drx, const double* dry,
                        const double* drz, const double* d2, double* out);
void orc_lj_force(int64_t n, const double* x, const double* y, const double* z,
                  const int64_t* off, const int32_t* nbr, const int8_t* img, const double L[3],
                  const orc_lj_params* p, double* fx, double* fy, double* fz, double* ep, double* vir);
void orc_lj_multi_force(int64_t n, const double* x, const double* y, const double* z, const uint8_t* type,
                        const int64_t* off, const int32_t* nbr, const int8_t* img, const double L[3],
                        const orc_lj_multi_params* p, double* fx, double* fy, double* fz, double* ep,
                        double* vir);
double orc_lj_direct(int64_t n, const double* x, const double* y, const double* z, const double lo[3],
                     const double hi[3], const orc_lj_params* p, double* fx, double* fy, double* fz);

void orc_eam_spline(int n, double delta, const double* f, double* spline);
double orc_eam_rho(const orc_eam_tables* t, double r, int itype, int jtype);
void orc_eam_embed_one(const orc_eam_tables* t, double rho, int itype, double* phi, double* fp);
void orc_eam_pair_force(const orc_eam_tables* t, double r, double fpi, double fpj, int itype, int jtype,
                        double* fpair, double* phi);
void orc_eam_density(int64_t n, const double* x, const double* y, const double* z, const uint8_t* type,
                     const int64_t* off, const int32_t* nbr, const int8_t* img, const double L[3],
                     const orc_eam_tables* t, double rcut, double* rho);
void orc_eam_embed(int64_t n, const uint8_t* type, const orc_eam_tables* t, double* rho_dEmb, double* ep);
void orc_eam_force(int64_t n, const double* x, const double* y, const double* z, const uint8_t* type,
                   const int64_t* off, const int32_t* nbr, const int8_t* img, const double L[3],
                   const orc_eam_tables* t, double rcut, const double* fp, double* fx, double* fy,
                   double* fz, double* ep, double* vir);

void orc_push_f_v_r(int64_t n, double* x, double* y, double* z, const double* vx, const double* vy,
                    const double* vz, const double* ax, const double* ay, const double* az, double dt,
                    double dt_scale);
void orc_push_f_v(int64_t n, double* vx, double* vy, double* vz, const double* ax, const double* ay,
                  const double* az, double dt, double dt_scale);
void orc_push_min(int64_t n, double* x, double* y, double* z, double* ax, double* ay, double* az,
                  const uint8_t* type, const double* masses, double dt, double dt_scale, double tolF);
void orc_force_to_accel(int64_t n, double* fx, double* fy, double* fz, const uint8_t* type,
                        const double* masses);
void orc_thermo(int64_t n, const double* vx, const double* vy, const double* vz, const double* ep,
                const double* vir, const uint8_t* type, const double* masses, double out[27]);

/* Parameter adjoint of the force-matching + energy loss for one single-element
 * configuration, in eV units (tables with conv = 1):
 *   L = wF * sum_i |F_i - F*_i|^2 + wE * sum_i (E_i - E*_i)^2
 * d-tables: for each parameter, the 7-coefficient spline of the derivative of
 * the tabulated knot values (the spline map is linear in the knot values).
 * Returns L; adds dL/dtheta into grad[nparam]; writes F (3n, xyz
 * interleaved) and E (n) when given. */
typedef struct {
  int nparam, pad_;
  const double* dfrho; /* nparam x (nrho+1) x 8 */
  const double* drhor; /* nparam x (nr+1) x 8 */
  const double* dz2r;  /* nparam x (nr+1) x 8 */
} orc_eam_dtables;

double orc_eam_loss_grad(int64_t n, const double* x, const double* y, const double* z, const int64_t* off,
                         const int32_t* nbr, const int8_t* img, const double L[3], const orc_eam_tables* t,
                         double rcut, const orc_eam_dtables* d, const double* Ft, const double* Et, double wF,
                         double wE, double* grad, double* F, double* E);

int orc_run_nve(int64_t n, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                double* ax, double* ay, double* az, double* ep, const uint8_t* type, const uint64_t* id,
                const double* masses, const double lo[3], const double hi[3], int pot_kind,
                const void* pot, double skin, double dt, int nsteps, int rebuild_every,
                double* thermo_out);
/* The same continuing from the given accelerations (ax, ay, az as the last
 * force pass left them, e.g. before the domain was rescaled): the first step
 * pushes with them instead of recomputing the forces first.  The step-0
 * thermo row then has the given state's kinetic terms and zero potential
 * terms. */
int orc_run_nve_from(int64_t n, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                     double* ax, double* ay, double* az, double* ep, const uint8_t* type, const uint64_t* id,
                     const double* masses, const double lo[3], const double hi[3], int pot_kind,
                     const void* pot, double skin, double dt, int nsteps, int rebuild_every,
                     double* thermo_out);

/* The minimisation graph: forces, clipped push r += a*dt^2/2
 * (push_vec3_2nd_order_xform_minimization.cpp L116-149), list rebuilt every
 * rebuild_every steps.  Returns 0, or a negative code as orc_run_nve. */
int orc_run_minimize(int64_t n, double* x, double* y, double* z, double* ax, double* ay, double* az,
                     double* ep, const uint8_t* type, const uint64_t* id, const double* masses,
                     const double lo[3], const double hi[3], int pot_kind, const void* pot, double skin,
                     double dt, double tolF, int nsteps, int rebuild_every);

/* list builds done by the last orc_run_nve / orc_run_minimize call (the
 * initial build included); rebuild_every == -1 in either selects the
 * displacement trigger: rebuild when some atom moved more than skin/2. */
int64_t orc_last_list_builds(void);

void orc_ej_phi(const orc_johnson_params* p, double r, double* phi, double* dphi);
void orc_ej_rho(const orc_johnson_params* p, double r, double* rho, double* drho);
void orc_ej_embed(const orc_johnson_params* p, double rho, double* f, double* df);
void orc_sc_phi(const orc_sutton_chen_params* p, double r, double* phi, double* dphi);
void orc_sc_rho(const orc_sutton_chen_params* p, double r, double* rho, double* drho);
void orc_sc_embed(const orc_sutton_chen_params* p, double rho, double* f, double* df);
/* Both passes of sutton_chen_force over a CSR list; fp receives F'(rho_i). */
void orc_sc_forces(int64_t n, const double* x, const double* y, const double* z, const int64_t* off,
                   const int32_t* nbr, const int8_t* img, const double L[3], const orc_sutton_chen_params* p,
                   double rcut, double* fp, double* fx, double* fy, double* fz, double* ep, double* vir);
/* Both passes of johnson_force over a CSR list; fp receives F'(rho_i). */
void orc_ej_forces(int64_t n, const double* x, const double* y, const double* z, const int64_t* off,
                   const int32_t* nbr, const int8_t* img, const double L[3], const orc_johnson_params* p,
                   double rcut, double* fp, double* fx, double* fy, double* fz, double* ep, double* vir);

/* lj_compute_force force-matching + energy loss and d(loss)/d(epsilon, sigma)
 * (targets: forces and per-atom energies); returns the loss. */
double orc_lj_loss_grad(int64_t n, const double* x, const double* y, const double* z, const int64_t* off,
                        const int32_t* nbr, const int8_t* img, const double L[3], const orc_lj_params* p,
                        const double* fxt, const double* fyt, const double* fzt, const double* et, double wF,
                        double wE, double grad[2]);

int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
